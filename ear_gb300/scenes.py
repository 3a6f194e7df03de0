"""Seeded synthetic scenes for the benchmark configurations.

The reference ships no scene files (its examples are Blender .blend files),
so every workload here is generated from a seed with the sizes the
benchmark names.  Each generator returns a ``Workload``: merged triangles
in MESH-block order, one material id per triangle, the MAT blocks, the
source, the recorders and the render settings.

  shoebox()       10x7x4 m room, 12 triangles, 1 specular material, mono
  relief_hall()   30x20x12 m room, heightfield walls, 20,000 triangles,
                  8 materials round-robin, stereo recorder
  cathedral()     60x25 m nave, 40 columns (32-sided, r 0.6 m), ribbed vault
                  of 1.2 M triangles, 2,000,000 triangles, 12 materials,
                  1 stereo + 8 mono recorders
  sweep_rooms()   16 convex rooms with 500..200,000 triangles, 16
                  source/listener pairs each, 24-keyframe source paths
  inverse_shoebox() shoebox geometry with 8 materials round-robin
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from .scene import Material, Recorder, Source

SR = 44100


@dataclass
class Workload:
    name: str
    vertices: np.ndarray          # (n, 9) float32
    material_ids: np.ndarray      # (n,) int32
    materials: List[Material]
    source: Source
    recorders: List[Recorder]
    render: dict = field(default_factory=dict)  # num_rays, max_bounces, num_bins, cutoff, ...
    block_sizes: Optional[List[int]] = None     # triangles per MESH block (file order)

    @property
    def num_triangles(self) -> int:
        return int(self.vertices.shape[0])

    @property
    def num_tracks(self) -> int:
        return sum(r.tracks for r in self.recorders)


def _quad(a, b, c, d):
    """Two triangles of quad a-b-c-d (the exporter's split, src export
    blender/render_EAR/__init__.py:259: [0,1,2], [0,2,3])."""
    return [np.concatenate([a, b, c]), np.concatenate([a, c, d])]


def box_triangles(lx, ly, lz) -> np.ndarray:
    """Axis-aligned box [0,lx]x[0,ly]x[0,lz] as 12 triangles (6 quads),
    wound with outward normals like a Blender cube (so Mesh::Volume is
    positive)."""
    P = lambda x, y, z: np.array([x, y, z], np.float32)
    q = []
    q += _quad(P(0, 0, 0), P(0, ly, 0), P(lx, ly, 0), P(lx, 0, 0))        # floor
    q += _quad(P(0, 0, lz), P(lx, 0, lz), P(lx, ly, lz), P(0, ly, lz))    # ceiling
    q += _quad(P(0, 0, 0), P(lx, 0, 0), P(lx, 0, lz), P(0, 0, lz))        # y = 0
    q += _quad(P(0, ly, 0), P(0, ly, lz), P(lx, ly, lz), P(lx, ly, 0))    # y = ly
    q += _quad(P(0, 0, 0), P(0, 0, lz), P(0, ly, lz), P(0, ly, 0))        # x = 0
    q += _quad(P(lx, 0, 0), P(lx, ly, 0), P(lx, ly, lz), P(lx, 0, lz))    # x = lx
    return np.stack(q).astype(np.float32)


def shoebox(num_rays: int = 100_000, seed: int = 0) -> Workload:
    """10x7x4 m shoebox, 12 triangles, one specular material with
    absorption 0.10/0.20/0.30 (reflection 0.9/0.8/0.7), point source at
    (2,3.5,1.5), mono recorder at (7,3.5,1.5), 2 s at 44.1 kHz, cut-off
    1e-6 or 50 reflections, no air absorption, dry level 1."""
    v = box_triangles(10.0, 7.0, 4.0)
    mats = [Material(reflection=(0.9, 0.8, 0.7), specularity=(1.0, 1.0, 1.0), name="specular")]
    return Workload(
        name="shoebox-12tri-mono",
        vertices=v, material_ids=np.zeros(len(v), np.int32), materials=mats,
        source=Source(location=np.array([2.0, 3.5, 1.5], np.float32)),
        recorders=[Recorder(location=np.array([7.0, 3.5, 1.5], np.float32))],
        render=dict(num_rays=num_rays, max_bounces=50, num_bins=2 * SR, cutoff=1e-6,
                    air_absorption=(0.0, 0.0, 0.0), dry=1.0, seed=seed),
        block_sizes=[len(v)])


def inverse_shoebox(num_rays: int = 1_000_000, seed: int = 0, hidden_seed: int = 7):
    """Shoebox geometry with 8 materials assigned round-robin; returns the
    workload (initial guess: absorption 0.2, refraction 0.05, spec 0.5) and
    the hidden (absorption, refraction) arrays of shape (8, 3) drawn from
    ``hidden_seed``."""
    base = shoebox(num_rays=num_rays, seed=seed)
    rng = np.random.default_rng(hidden_seed)
    hid_abs = rng.uniform(0.05, 0.5, size=(8, 3)).astype(np.float32)
    hid_refr = rng.uniform(0.0, 0.1, size=(8, 3)).astype(np.float32)
    mats = [Material(reflection=(0.75, 0.75, 0.75), refraction=(0.05, 0.05, 0.05),
                     specularity=(0.5, 0.5, 0.5), name=f"m{i}") for i in range(8)]
    base.materials = mats
    base.material_ids = (np.arange(base.num_triangles) % 8).astype(np.int32)
    base.name = "shoebox-8mat-inverse"
    return base, hid_abs, hid_refr


def _value_noise(rng, shape_cells, u, v):
    """Smooth value noise on a lattice (cosine-interpolated random values)."""
    gx, gy = shape_cells
    lat = rng.uniform(-1.0, 1.0, size=(gx + 2, gy + 2)).astype(np.float64)
    x = u * gx
    y = v * gy
    i = np.floor(x).astype(int)
    j = np.floor(y).astype(int)
    fx = x - i
    fy = y - j
    sx = (1 - np.cos(np.pi * fx)) * 0.5
    sy = (1 - np.cos(np.pi * fy)) * 0.5
    a = lat[i, j] * (1 - sx) + lat[i + 1, j] * sx
    b = lat[i, j + 1] * (1 - sx) + lat[i + 1, j + 1] * sx
    return a * (1 - sy) + b * sy


def _grid_wall(origin, eu, ev, normal, nu, nv, rng, amplitude, cells=(6, 4)):
    """A displaced nu x nv grid of quads spanning origin + s*eu + t*ev; the
    displacement (along ``normal``, pointing into the room) tapers to zero
    on the border so walls meet exactly at the room edges.  Triangles are
    wound with their normals facing out of the room."""
    s = np.linspace(0.0, 1.0, nu + 1)
    t = np.linspace(0.0, 1.0, nv + 1)
    S, T = np.meshgrid(s, t, indexing="ij")
    h = _value_noise(rng, cells, S, T) + 0.5 * _value_noise(rng, (cells[0] * 3, cells[1] * 3), S, T)
    h = h / 1.5 * amplitude * np.sin(np.pi * S) * np.sin(np.pi * T)
    P = (origin[None, None, :] + S[..., None] * eu[None, None, :] + T[..., None] * ev[None, None, :]
         + h[..., None] * normal[None, None, :])
    a = P[:-1, :-1].reshape(-1, 3)
    b = P[1:, :-1].reshape(-1, 3)
    c = P[1:, 1:].reshape(-1, 3)
    d = P[:-1, 1:].reshape(-1, 3)
    t1 = np.concatenate([a, c, b], 1)
    t2 = np.concatenate([a, d, c], 1)
    return np.stack([t1, t2], 1).reshape(-1, 9)


def relief_hall(num_rays: int = 10_000_000, seed: int = 1) -> Workload:
    """30x20x12 m hall whose six walls are heightfield grids (value noise,
    amplitude 0.3 m): 60x40 quads on floor and ceiling, 60x26 on the long
    walls, 40x26 on the end walls = 20,000 triangles, round-robin over 8
    materials with absorption U[0.02,0.6], refraction U[0,0.1] (seed 1),
    specularity U[0.1,0.9].  One source, one stereo recorder (head size
    0.18 m), 3 s histograms, 200 reflections, exporter-default air
    absorption 0.01/0.02/0.05 per metre."""
    rng = np.random.default_rng(seed)
    L, W, H = 30.0, 20.0, 12.0
    f = lambda *x: np.array(x, np.float64)
    walls = [
        _grid_wall(f(0, 0, 0), f(L, 0, 0), f(0, W, 0), f(0, 0, 1), 60, 40, rng, 0.3),      # floor
        _grid_wall(f(0, 0, H), f(0, W, 0), f(L, 0, 0), f(0, 0, -1), 40, 60, rng, 0.3),     # ceiling
        _grid_wall(f(0, 0, 0), f(0, 0, H), f(L, 0, 0), f(0, 1, 0), 26, 60, rng, 0.3),      # y = 0
        _grid_wall(f(0, W, 0), f(L, 0, 0), f(0, 0, H), f(0, -1, 0), 60, 26, rng, 0.3),     # y = W
        _grid_wall(f(0, 0, 0), f(0, W, 0), f(0, 0, H), f(1, 0, 0), 40, 26, rng, 0.3),      # x = 0
        _grid_wall(f(L, 0, 0), f(0, 0, H), f(0, W, 0), f(-1, 0, 0), 26, 40, rng, 0.3),     # x = L
    ]
    v = np.concatenate(walls, 0).astype(np.float32)
    assert v.shape[0] == 20000, v.shape
    mrng = np.random.default_rng(seed)
    absorb = mrng.uniform(0.02, 0.6, size=(8, 3))
    refr = mrng.uniform(0.0, 0.1, size=(8, 3))
    spec = mrng.uniform(0.1, 0.9, size=(8, 3))
    mats = [Material(reflection=tuple((1.0 - absorb[i] - refr[i]).tolist()),
                     refraction=tuple(refr[i].tolist()), specularity=tuple(spec[i].tolist()),
                     name=f"relief{i}") for i in range(8)]
    ids = (np.arange(v.shape[0]) % 8).astype(np.int32)
    rec = Recorder(location=np.array([21.0, 9.0, 1.7], np.float32), channels=2,
                   right_ear=np.array([0.0, -1.0, 0.0], np.float32), head_size=0.18,
                   head_absorption=(0.1, 0.3, 0.9))
    return Workload(
        name="relief-hall-20k-stereo", vertices=v, material_ids=ids, materials=mats,
        source=Source(location=np.array([7.5, 11.0, 1.8], np.float32)),
        recorders=[rec],
        render=dict(num_rays=num_rays, max_bounces=200, num_bins=3 * SR, cutoff=1e-8,
                    air_absorption=(0.01, 0.02, 0.05), dry=1.0, seed=seed),
        block_sizes=None)


def _cylinder(cx, cy, r, z0, z1, sides, segs):
    ang = np.linspace(0.0, 2 * np.pi, sides + 1)
    z = np.linspace(z0, z1, segs + 1)
    A, Z = np.meshgrid(ang, z, indexing="ij")
    P = np.stack([cx + r * np.cos(A), cy + r * np.sin(A), Z], -1)
    a = P[:-1, :-1].reshape(-1, 3)
    b = P[1:, :-1].reshape(-1, 3)
    c = P[1:, 1:].reshape(-1, 3)
    d = P[:-1, 1:].reshape(-1, 3)
    tris = np.stack([np.concatenate([a, b, c], 1), np.concatenate([a, c, d], 1)], 1).reshape(-1, 9)
    top = np.array([cx, cy, z1])
    cap = [np.concatenate([P[i, -1], P[i + 1, -1], top]) for i in range(sides)]
    return np.concatenate([tris, np.array(cap)], 0)


def _plane_grid(origin, eu, ev, nu, nv):
    """Flat nu x nv grid; eu x ev points into the room, triangles face out."""
    s = np.linspace(0.0, 1.0, nu + 1)
    t = np.linspace(0.0, 1.0, nv + 1)
    S, T = np.meshgrid(s, t, indexing="ij")
    P = origin[None, None, :] + S[..., None] * eu[None, None, :] + T[..., None] * ev[None, None, :]
    a = P[:-1, :-1].reshape(-1, 3)
    b = P[1:, :-1].reshape(-1, 3)
    c = P[1:, 1:].reshape(-1, 3)
    d = P[:-1, 1:].reshape(-1, 3)
    return np.stack([np.concatenate([a, c, b], 1), np.concatenate([a, d, c], 1)], 1).reshape(-1, 9)


def cathedral(num_rays: int = 100_000_000, seed: int = 5, total: int = 2_000_000) -> Workload:
    """Cathedral-like nave: 60x25 m floor, 18 m walls, a ribbed pointed
    vault tessellated to 1.2 M triangles, 40 columns (two rows of 20,
    32-sided cylinders of radius 0.6 m), gable walls closing the vault ends,
    and floor/wall grids sized so the scene has exactly ``total`` triangles;
    12 materials; one stereo and eight mono recorders; 4 s histograms, 300
    reflections."""
    rng = np.random.default_rng(seed)
    L, W, Hw, rise = 60.0, 25.0, 18.0, 7.0
    f = lambda *x: np.array(x, np.float64)
    parts, mids = [], []

    def add(tris, mat):
        parts.append(np.asarray(tris, np.float64))
        mids.append(np.full(len(tris), mat, np.int32))

    # ribbed pointed vault: 1000 x 600 quads = 1.2 M triangles
    nu, nv = 1000, 600
    xs = np.linspace(0.0, L, nu + 1)
    ys = np.linspace(0.0, W, nv + 1)
    X, Y = np.meshgrid(xs, ys, indexing="ij")
    prof = rise * np.sin(np.pi * Y / W) ** 0.7
    ribs = 0.35 * np.exp(-((np.mod(X, 5.0) - 2.5) / 0.25) ** 2)  # transverse ribs every 5 m
    diag = 0.25 * np.exp(-((np.abs(np.mod(X, 5.0) - 2.5) * W / 5.0 - np.abs(Y - W / 2)) / 0.3) ** 2)
    Z = Hw + prof - ribs - diag
    P = np.stack([X, Y, Z], -1)
    a = P[:-1, :-1].reshape(-1, 3)
    b = P[:-1, 1:].reshape(-1, 3)
    c = P[1:, 1:].reshape(-1, 3)
    d = P[1:, :-1].reshape(-1, 3)
    vault = np.stack([np.concatenate([a, c, b], 1), np.concatenate([a, d, c], 1)], 1).reshape(-1, 9)
    # rib quads get their own material
    rq = ((ribs + diag)[:-1, :-1] > 0.05).reshape(-1)
    vm = np.where(np.repeat(rq, 2), 10, 9).astype(np.int32)
    parts.append(vault)
    mids.append(vm)
    # gables closing the vault at x = 0 and x = L (quads between the
    # springing line and the vault profile)
    for x0 in (0.0, L):
        zprof = Z[0 if x0 == 0.0 else -1]
        g = []
        for j in range(nv):
            p0 = f(x0, ys[j], Hw)
            p1 = f(x0, ys[j + 1], Hw)
            p2 = f(x0, ys[j + 1], zprof[j + 1])
            p3 = f(x0, ys[j], zprof[j])
            g += _quad(p0, p3, p2, p1) if x0 == 0.0 else _quad(p0, p1, p2, p3)
        add(np.array(g), 8)
    # 40 columns: two rows of 20, 32 sides, 100 segments, capped
    for row_y in (6.5, W - 6.5):
        for k in range(20):
            cx = 1.5 + k * (57.0 / 19.0)
            add(_cylinder(cx, row_y, 0.6, 0.0, Hw, 32, 100), 6 + (k % 2))
    used = sum(len(p) for p in parts)
    remain = total - used
    # floor a x b quads, 4 walls with h rows: 2ab + 4h(a + b) triangles
    best = None
    for h in range(100, 220):
        for a_ in range(300, 900):
            rest = remain - 4 * h * a_
            if rest <= 0:
                break
            # 2 a b + 4 h b = rest  ->  b = rest / (2a + 4h)
            den = 2 * a_ + 4 * h
            if rest % den == 0:
                b_ = rest // den
                if 100 <= b_ <= 600:
                    cand = (abs(a_ / b_ - L / W) + abs(h / b_ - Hw / W), a_, b_, h)
                    if best is None or cand < best:
                        best = cand
    if best is None:
        raise RuntimeError("no exact tessellation for the requested triangle count")
    _, na, nb, nh = best
    add(_plane_grid(f(0, 0, 0), f(L, 0, 0), f(0, W, 0), na, nb), 0)            # floor
    add(_plane_grid(f(0, 0, 0), f(0, 0, Hw), f(L, 0, 0), nh, na), 1)           # y = 0
    add(_plane_grid(f(0, W, 0), f(L, 0, 0), f(0, 0, Hw), na, nh), 2)           # y = W
    add(_plane_grid(f(0, 0, 0), f(0, W, 0), f(0, 0, Hw), nb, nh), 3)           # x = 0
    add(_plane_grid(f(L, 0, 0), f(0, 0, Hw), f(0, W, 0), nh, nb), 4)           # x = L
    v = np.concatenate(parts, 0).astype(np.float32)
    ids = np.concatenate(mids, 0)
    assert v.shape[0] == total, (v.shape, total)
    # 12 materials: stone floor, walls, glazing-like end wall, columns,
    # vault webs and ribs, plus three spare variants used by small patches
    mats = []
    for i in range(12):
        absorb = rng.uniform(0.02, 0.35, 3)
        refr = rng.uniform(0.0, 0.05, 3) if i in (4, 8) else None
        refl = 1.0 - absorb - (refr if refr is not None else 0.0)
        spec = rng.uniform(0.2, 0.9, 3)
        mats.append(Material(reflection=tuple(refl.tolist()),
                             refraction=None if refr is None else tuple(refr.tolist()),
                             specularity=tuple(spec.tolist()), name=f"cath{i}"))
    # spare materials 5 and 11 on a few floor patches
    patch = rng.choice(2 * na * nb, size=2000, replace=False) + used
    ids[patch[:1000]] = 5
    ids[patch[1000:]] = 11
    recs = [Recorder(location=np.array([40.0, 12.5, 1.7], np.float32), channels=2,
                     right_ear=np.array([0.0, -1.0, 0.0], np.float32), head_size=0.18,
                     head_absorption=(0.1, 0.3, 0.9))]
    for k in range(8):
        recs.append(Recorder(location=np.array([12.0 + 6.0 * k, 3.0 + 19.0 * (k % 2), 1.5],
                                               np.float32)))
    return Workload(
        name="cathedral-2M-stereo+8mono", vertices=v, material_ids=ids.astype(np.int32),
        materials=mats, source=Source(location=np.array([5.0, 12.5, 2.0], np.float32)),
        recorders=recs,
        render=dict(num_rays=num_rays, max_bounces=300, num_bins=4 * SR, cutoff=1e-8,
                    air_absorption=(0.01, 0.02, 0.05), dry=1.0, seed=seed),
        block_sizes=None)


def small_test_room(seed: int = 3, n_side: int = 4) -> Workload:
    """A small closed room with displaced walls (a few hundred triangles),
    two materials with refraction, a stereo and a mono recorder -- sized so
    the brute-force CPU restatement finishes in seconds."""
    rng = np.random.default_rng(seed)
    L, W, H = 8.0, 6.0, 3.5
    f = lambda *x: np.array(x, np.float64)
    n = n_side
    walls = [
        _grid_wall(f(0, 0, 0), f(L, 0, 0), f(0, W, 0), f(0, 0, 1), 2 * n, n + 1, rng, 0.2, (3, 2)),
        _grid_wall(f(0, 0, H), f(0, W, 0), f(L, 0, 0), f(0, 0, -1), n + 1, 2 * n, rng, 0.2, (2, 3)),
        _grid_wall(f(0, 0, 0), f(0, 0, H), f(L, 0, 0), f(0, 1, 0), n, 2 * n, rng, 0.2, (2, 3)),
        _grid_wall(f(0, W, 0), f(L, 0, 0), f(0, 0, H), f(0, -1, 0), 2 * n, n, rng, 0.2, (3, 2)),
        _grid_wall(f(0, 0, 0), f(0, W, 0), f(0, 0, H), f(1, 0, 0), n + 1, n, rng, 0.2, (2, 2)),
        _grid_wall(f(L, 0, 0), f(0, 0, H), f(0, W, 0), f(-1, 0, 0), n, n + 1, rng, 0.2, (2, 2)),
    ]
    v = np.concatenate(walls, 0).astype(np.float32)
    # an occluding pillar so visibility queries are not all trivially true
    pillar = box_triangles(0.6, 0.6, 2.5) + np.tile(np.array([3.7, 2.7, 0.0], np.float32), 3)
    v = np.concatenate([v, pillar], 0)
    mats = [Material(reflection=(0.85, 0.7, 0.6), refraction=(0.05, 0.1, 0.15),
                     specularity=(0.2, 0.5, 0.8), name="plaster"),
            Material(reflection=(0.5, 0.6, 0.7), specularity=(0.9, 0.7, 0.3), name="wood"),
            Material(reflection=(0.0, 0.0, 0.0), refraction=(0.00005, 0.2, 0.5), name="curtain")]
    ids = (np.arange(v.shape[0]) % 3).astype(np.int32)
    recs = [Recorder(location=np.array([6.0, 4.5, 1.6], np.float32), channels=2,
                     right_ear=np.array([0.0, -1.0, 0.0], np.float32), head_size=0.2,
                     head_absorption=(0.1, 0.3, 0.9)),
            Recorder(location=np.array([5.5, 1.2, 1.2], np.float32))]
    return Workload(
        name="small-test-room", vertices=v, material_ids=ids, materials=mats,
        source=Source(location=np.array([1.5, 2.0, 1.7], np.float32), gain=0.8),
        recorders=recs,
        render=dict(num_rays=2000, max_bounces=60, num_bins=SR, cutoff=1e-6,
                    air_absorption=(0.01, 0.02, 0.05), dry=1.0, seed=seed))


# ------------------------------------------------------------------ sweep
@dataclass
class SweepRoom:
    """One room of the batched sweep: a convex polyhedron with subdivided
    faces, its materials, and source / listener pairs (the source animated
    over keyframes)."""
    name: str
    vertices: np.ndarray          # (n, 9) float32, outward normals
    material_ids: np.ndarray      # (n,) int32
    materials: List[Material]
    sources: List[Source]         # per pair, location (keyframes, 3)
    listeners: List[Recorder]     # per pair, mono
    halfspaces: np.ndarray        # (faces, 4): n.x + d <= 0 inside

    @property
    def num_triangles(self) -> int:
        return int(self.vertices.shape[0])


def _subdivide(tris: np.ndarray, levels: int) -> np.ndarray:
    """Midpoint 4-split of every triangle, `levels` times (stays planar,
    keeps the winding)."""
    t = tris.reshape(-1, 3, 3)
    for _ in range(levels):
        a, b, c = t[:, 0], t[:, 1], t[:, 2]
        ab, bc, ca = (a + b) * 0.5, (b + c) * 0.5, (c + a) * 0.5
        t = np.stack([np.stack([a, ab, ca], 1), np.stack([ab, b, bc], 1),
                      np.stack([ca, bc, c], 1), np.stack([ab, bc, ca], 1)], 1).reshape(-1, 3, 3)
    return t.reshape(-1, 9)


def _inside(h: np.ndarray, p: np.ndarray, margin: float) -> bool:
    return bool(np.all(h[:, :3] @ p + h[:, 3] <= -margin))


def convex_room(rng, target_tris: int, n_mats: int, name: str = "room") -> SweepRoom:
    """Random convex polyhedron: the hull of points on a random ellipsoid
    (half-axes 4..15 m), faces 4-split until the triangle count is near
    ``target_tris``; one random material per hull face."""
    from scipy.spatial import ConvexHull

    levels = 0
    while target_tris / (4 ** levels) > 2000:
        levels += 1
    faces = max(8, int(round(target_tris / (4 ** levels))))
    npts = faces // 2 + 2
    radii = rng.uniform(4.0, 15.0, 3)
    d = rng.standard_normal((npts, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    pts = d * radii + radii  # corner of the bounding box at the origin
    hull = ConvexHull(pts)
    centre = pts.mean(0)
    simp = hull.simplices.copy()
    P = pts[simp]  # (F, 3, 3)
    n = np.cross(P[:, 1] - P[:, 0], P[:, 2] - P[:, 0])
    flip = np.einsum("ij,ij->i", n, P.mean(1) - centre) < 0
    simp[flip] = simp[flip][:, [0, 2, 1]]
    tris = pts[simp].reshape(-1, 9)
    face_mat = rng.integers(0, n_mats, len(simp))
    v = _subdivide(tris, levels).astype(np.float32)
    ids = np.repeat(face_mat, 4 ** levels).astype(np.int32)
    absorb = rng.uniform(0.02, 0.6, size=(n_mats, 3))
    refr = rng.uniform(0.0, 0.1, size=(n_mats, 3))
    spec = rng.uniform(0.1, 0.9, size=(n_mats, 3))
    mats = [Material(reflection=tuple((1.0 - absorb[i] - refr[i]).tolist()),
                     refraction=tuple(refr[i].tolist()), specularity=tuple(spec[i].tolist()),
                     name=f"{name}-m{i}") for i in range(n_mats)]
    return SweepRoom(name=name, vertices=v, material_ids=ids, materials=mats, sources=[],
                     listeners=[], halfspaces=hull.equations.astype(np.float64))


def _point_inside(rng, room: SweepRoom, margin: float) -> np.ndarray:
    lo = room.vertices.reshape(-1, 3).min(0)
    hi = room.vertices.reshape(-1, 3).max(0)
    for _ in range(100000):
        p = rng.uniform(lo, hi)
        if _inside(room.halfspaces, p, margin):
            return p
    raise RuntimeError("no interior point found")


def sweep_rooms(num_rooms: int = 16, pairs_per_room: int = 16, keyframes: int = 24,
                path_length: float = 5.0, min_tris: int = 500, max_tris: int = 200_000,
                seed: int = 3):
    """The batched sweep: ``num_rooms`` convex rooms whose triangle counts
    are log-uniform in [min_tris, max_tris], 4-8 materials each, and
    ``pairs_per_room`` source / listener pairs placed uniformly inside
    (0.5 m from the walls); each source moves along a random straight
    ``path_length`` m path sampled at ``keyframes`` keyframes.  Render
    settings: 2 s mono histograms, 3 bands, 200 reflections, cut-off 1e-8,
    1e6 rays per pair-frame.  Returns (rooms, render settings)."""
    rng = np.random.default_rng(seed)
    rooms = []
    for r in range(num_rooms):
        target = int(round(np.exp(rng.uniform(np.log(min_tris), np.log(max_tris)))))
        room = convex_room(rng, target, int(rng.integers(4, 9)), name=f"sweep{r}")
        for _ in range(pairs_per_room):
            for _try in range(1000):
                a = _point_inside(rng, room, 0.5)
                u = rng.standard_normal(3)
                u /= np.linalg.norm(u)
                b = a + path_length * u
                if _inside(room.halfspaces, b, 0.5):
                    break
            else:
                raise RuntimeError("no source path fits inside the room")
            t = np.linspace(0.0, 1.0, keyframes)[:, None]
            room.sources.append(Source(location=((1 - t) * a + t * b).astype(np.float32)))
            room.listeners.append(Recorder(location=_point_inside(rng, room, 0.5).astype(np.float32)))
        rooms.append(room)
    render = dict(num_rays=1_000_000, max_bounces=200, num_bins=2 * SR, cutoff=1e-8,
                  air_absorption=(0.01, 0.02, 0.05), dry=1.0, seed=seed)
    return rooms, render

"""Python host side of the ray-tracing core.

``Scene`` mirrors the reference's ``Scene`` class (src/Scene.h:42-79):
meshes are merged in insertion order (``addMesh``, src/Scene.cpp:103-106),
materials are registered by name (``addMaterial``, :107-109), listeners and
sources are appended, and ``Render`` has the argument list of
``Scene::Render`` (src/Scene.h:77).  Underneath, everything goes through the
C ABI (``ear_gb300._native``) to the sm_103a kernels; there is no CPU path.

``Tracer`` is the lower-level handle: one uploaded scene with its LBVH,
rendering all bands of one (source, keyframe) context per call.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np

from . import _native as N


@dataclass
class Material:
    """A MAT block (src/Material.cpp:26-72): per-band reflection, optional
    refraction and specularity triplets."""
    reflection: Sequence[float]
    refraction: Optional[Sequence[float]] = None
    specularity: Optional[Sequence[float]] = None
    name: str = ""

    def to_c(self) -> N.EarMaterial:
        m = N.EarMaterial()
        m.reflection[:] = [float(x) for x in self.reflection]
        if self.refraction is not None:
            m.refraction[:] = [float(x) for x in self.refraction]
            m.has_refraction = 1
        if self.specularity is not None:
            m.specularity[:] = [float(x) for x in self.specularity]
            m.has_specularity = 1
        return m


def _frames(x, n_frames: Optional[int] = None) -> np.ndarray:
    a = np.asarray(x, dtype=np.float32)
    if a.ndim == 1:
        a = a[None, :]
    return a


@dataclass
class Recorder:
    """OUT1 (mono) or OUT2 (stereo) block.  ``location`` / ``right_ear``
    are (3,) or (keyframes, 3) arrays (Animated<T>, src/Animated.h:66-108)."""
    location: np.ndarray
    channels: int = 1
    right_ear: np.ndarray = field(default_factory=lambda: np.array([1.0, 0.0, 0.0], np.float32))
    head_size: float = 0.2
    head_absorption: Sequence[float] = (0.1, 0.3, 0.9)
    filename: str = ""

    def at(self, keyframe: int) -> N.EarRecorder:
        loc = _frames(self.location)
        ear = _frames(self.right_ear)
        r = N.EarRecorder()
        r.channels = int(self.channels)
        r.location[:] = [float(v) for v in loc[keyframe if keyframe >= 0 and len(loc) > 1 else 0]]
        r.right_ear[:] = [float(v) for v in ear[keyframe if keyframe >= 0 and len(ear) > 1 else 0]]
        r.head_size = float(self.head_size)
        r.head_absorption[:] = [float(v) for v in self.head_absorption]
        return r

    @property
    def tracks(self) -> int:
        return 2 if self.channels == 2 else 1


@dataclass
class Source:
    """SSRC / 3SRC block: point location (or per-keyframe locations), gain,
    or an area emitter given as (n, 9) triangles."""
    location: np.ndarray = field(default_factory=lambda: np.zeros(3, np.float32))
    gain: float = 1.0
    emitter: Optional[np.ndarray] = None
    filename: str = ""
    offset: float = 0.0

    def at(self, keyframe: int):
        loc = _frames(self.location)
        s = N.EarSource()
        s.location[:] = [float(v) for v in loc[keyframe if keyframe >= 0 and len(loc) > 1 else 0]]
        s.gain = float(self.gain)
        keep = None
        if self.emitter is not None and len(self.emitter):
            keep = np.ascontiguousarray(self.emitter, dtype=np.float32).reshape(-1, 9)
            s.num_emitter_triangles = keep.shape[0]
            s.emitter_vertices = keep.ctypes.data_as(C.POINTER(C.c_float))
        return s, keep

    @property
    def is_mesh_source(self) -> bool:
        return self.emitter is not None and len(self.emitter) > 0


def recorders_at(recorders: Sequence[Recorder], keyframe: int):
    arr = (N.EarRecorder * max(1, len(recorders)))()
    for i, r in enumerate(recorders):
        arr[i] = r.at(keyframe)
    return arr


def make_params(*, seed=0, context=0, bands=(0, 1, 2), num_rays=1000, max_bounces=N.EAR_REFERENCE_MAX_BOUNCES,
                num_bins=3 * N.SAMPLE_RATE, cutoff=N.EAR_REFERENCE_CUTOFF, air_absorption=(0.0, 0.0, 0.0),
                dry=1.0, exact=False, raw=False, no_direct=False, stream=None,
                first_ray=0, traverse_budget=0) -> N.EarRenderParams:
    p = N.EarRenderParams()
    p.seed = int(seed)
    p.context = int(context) & 0xFFFFFFFF
    mask = 0
    for b in bands:
        mask |= 1 << int(b)
    p.bands_mask = mask
    p.num_rays = int(num_rays)
    p.max_bounces = int(max_bounces)
    p.num_bins = int(num_bins)
    p.cutoff = float(cutoff)
    p.air_absorption[:] = [float(x) for x in air_absorption]
    p.dry_level = float(dry)
    p.flags = (N.EAR_FLAG_EXACT if exact else 0) | (N.EAR_FLAG_RAW if raw else 0) | \
        (N.EAR_FLAG_NO_DIRECT if no_direct else 0)
    p.stream = stream
    p.first_ray = int(first_ray)
    p.traverse_budget = int(traverse_budget)
    return p


@dataclass
class RenderResult:
    hist: object              # numpy (tracks, 3, bins) or the caller's device tensor
    first_sample: np.ndarray  # (tracks, 3)
    last_sample: np.ndarray   # (tracks, 3)
    stats: dict
    raw_first_sample: Optional[np.ndarray] = None  # before 1/N scaling and direct sound
    raw_last_sample: Optional[np.ndarray] = None


class Tracer:
    """One scene uploaded to the GPU with its LBVH (ear_scene_create +
    ear_scene_build_bvh)."""

    def __init__(self, vertices, material_ids, materials: Sequence[Material], device: int = 0,
                 box_pad: float = -1.0, builder: str = "default", max_leaf: int = 0,
                 ploc_radius: int = 0, width: int = 0, visibility_order: int = 0,
                 visibility_map: int = 0):
        L = N.lib()
        self._v = np.ascontiguousarray(vertices, dtype=np.float32).reshape(-1, 9)
        self._m = np.ascontiguousarray(material_ids, dtype=np.int32).reshape(-1)
        if self._m.shape[0] != self._v.shape[0]:
            raise ValueError("one material id per triangle")
        self.materials = list(materials)
        mats = (N.EarMaterial * max(1, len(self.materials)))()
        for i, m in enumerate(self.materials):
            mats[i] = m.to_c()
        desc = N.EarSceneDesc()
        desc.num_triangles = self._v.shape[0]
        desc.vertices = self._v.ctypes.data_as(C.POINTER(C.c_float))
        desc.material_ids = self._m.ctypes.data_as(C.POINTER(C.c_int32))
        desc.num_materials = len(self.materials)
        desc.materials = mats
        desc.device = int(device)
        h = C.c_void_p()
        N.check(L.ear_scene_create(C.byref(desc), C.byref(h)))
        self._h = h
        self.build_bvh(box_pad=box_pad, builder=builder, max_leaf=max_leaf,
                       ploc_radius=ploc_radius, width=width, visibility_order=visibility_order,
                       visibility_map=visibility_map)

    def build_bvh(self, box_pad: float = -1.0, builder: str = "default", max_leaf: int = 0,
                  ploc_radius: int = 0, width: int = 0, visibility_order: int = 0,
                  visibility_map: int = 0) -> None:
        """(Re)build the BVH: builder "default", "lbvh" or "ploc"; traversal
        width 2, 4 or 0 (4-wide from 4096 triangles; a 4-wide tree deeper
        than 16 levels is not kept, and the binary tree serves); visibility_order 1
        nearest first, 2 farthest first, 0 automatic; visibility_map -1 off,
        8..4096 on with that many cells per cube-face edge, 0 automatic
        (listener visibility maps: visibility tests by direction lists
        around each recorder instead of tree traversals)."""
        opts = N.EarBvhOpts()
        opts.box_pad = float(box_pad)
        opts.max_leaf_size = int(max_leaf)
        opts.builder = {"default": N.EAR_BVH_DEFAULT, "lbvh": N.EAR_BVH_LBVH,
                        "ploc": N.EAR_BVH_PLOC}[builder]
        opts.ploc_radius = int(ploc_radius)
        opts.width = int(width)
        opts.visibility_order = int(visibility_order)
        opts.visibility_map = int(visibility_map)
        N.check(N.lib().ear_scene_build_bvh(self._h, C.byref(opts)))
        self._builder = builder

    @property
    def num_triangles(self) -> int:
        return int(self._v.shape[0])

    def info(self) -> dict:
        nt, nn, b, db = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        depth, pad = C.c_int32(), C.c_float()
        N.check(N.lib().ear_scene_info(self._h, C.byref(nt), C.byref(nn), C.byref(depth),
                                        C.byref(pad), C.byref(db)))
        return {"triangles": nt.value, "nodes": nn.value, "max_depth": depth.value,
                "box_pad": pad.value, "device_bytes": db.value,
                "builder": getattr(self, "_builder", "default"),
                "width": self.width}

    @property
    def width(self) -> int:
        """The tree the traversal uses: 2 (binary) or 4."""
        w = C.c_int32()
        N.check(N.lib().ear_scene_bvh_width(self._h, C.byref(w)))
        return w.value

    def sah_cost(self, width: int = 4, node_cost: float = 1.0,
                 triangle_cost: float = 1.0) -> float:
        """Surface-area-heuristic cost of the binary (2) or 4-wide (4) tree."""
        c = C.c_double()
        N.check(N.lib().ear_scene_sah_cost(self._h, int(width), float(node_cost),
                                           float(triangle_cost), C.byref(c)))
        return c.value

    def set_width(self, width: int) -> None:
        """Traverse the binary (2) or 4-wide (4) tree; no rebuild."""
        N.check(N.lib().ear_scene_set_bvh_width(self._h, int(width)))

    def render(self, source: Source, recorders: Sequence[Recorder], *, keyframe: int = -1,
               out=None, **kw) -> RenderResult:
        """Render every band of ``kw['bands']`` for one (source, keyframe).
        ``out`` may be a CUDA tensor of shape (tracks, 3, num_bins) float32,
        filled in place on the device."""
        src, _keep = source.at(keyframe)
        recs = recorders_at(recorders, keyframe)
        p = make_params(**kw)
        tracks = sum(r.tracks for r in recorders)
        first = np.zeros((max(tracks, 1), 3), np.int32)
        last = np.zeros((max(tracks, 1), 3), np.int32)
        h = N.EarHistograms()
        if out is None:
            hist = np.zeros((tracks, 3, p.num_bins), np.float32)
            h.data = hist.ctypes.data if tracks else first.ctypes.data
            h.on_device = 0
        else:
            hist = out
            if tuple(out.shape) != (tracks, 3, p.num_bins) or not out.is_contiguous():
                raise ValueError("out must be a contiguous (tracks, 3, num_bins) tensor")
            h.data = out.data_ptr()
            h.on_device = 1 if out.is_cuda else 0
            if out.is_cuda and p.stream is None:
                import torch
                p.stream = torch.cuda.current_stream(out.device).cuda_stream
        fdev = ldev = None
        if h.on_device:
            import torch
            fdev = torch.empty((max(tracks, 1), 3), dtype=torch.int32, device=out.device)
            ldev = torch.empty_like(fdev)
            h.first_sample, h.last_sample = fdev.data_ptr(), ldev.data_ptr()
        else:
            h.first_sample, h.last_sample = first.ctypes.data, last.ctypes.data
        raw_first = np.zeros((max(tracks, 1), 3), np.int32)
        raw_last = np.zeros((max(tracks, 1), 3), np.int32)
        if not h.on_device:
            h.raw_first_sample, h.raw_last_sample = raw_first.ctypes.data, raw_last.ctypes.data
        st = N.EarRenderStats()
        N.check(N.lib().ear_render(self._h, C.byref(src), recs, len(recorders), C.byref(p),
                                   C.byref(h), C.byref(st)))
        if fdev is not None:
            first, last = fdev.cpu().numpy(), ldev.cpu().numpy()
            raw_first = raw_last = None
        else:
            raw_first, raw_last = raw_first[:tracks], raw_last[:tracks]
        return RenderResult(hist, first[:tracks], last[:tracks], st.as_dict(), raw_first, raw_last)

    def set_materials(self, materials: Sequence[Material]) -> None:
        """Replace the MAT table (same count) without rebuilding the LBVH."""
        mats = (N.EarMaterial * max(1, len(materials)))()
        for i, m in enumerate(materials):
            mats[i] = m.to_c()
        N.check(N.lib().ear_scene_set_materials(self._h, mats, len(materials)))
        self.materials = list(materials)

    def render_adjoint(self, source: Source, recorders: Sequence[Recorder], d_hist, *,
                       first=None, last=None, raw_first=None, raw_last=None, keyframe: int = -1,
                       **kw):
        """Gradient of sum(d_hist * h) w.r.t. every material's per-band
        (absorption, refraction): an array (materials, 3, 2).  ``d_hist`` is a
        numpy array or CUDA tensor (tracks, 3, num_bins); the bookkeeping of
        the forward render (RenderResult.first/last/raw_*) is needed unless
        ``raw=True``."""
        src, _keep = source.at(keyframe)
        recs = recorders_at(recorders, keyframe)
        p = make_params(**kw)
        on_dev = hasattr(d_hist, "is_cuda") and d_hist.is_cuda
        if on_dev:
            d = d_hist.contiguous()
            ptr = d.data_ptr()
            if p.stream is None:
                import torch
                p.stream = torch.cuda.current_stream(d.device).cuda_stream
        else:
            d = np.ascontiguousarray(d_hist, np.float32)
            ptr = d.ctypes.data
        grad = np.zeros((len(self.materials), 3, 2), np.float64)
        keep = [np.ascontiguousarray(x, np.int32) if x is not None else None
                for x in (raw_first, raw_last, first, last)]
        ptrs = [k.ctypes.data if k is not None else None for k in keep]
        st = N.EarRenderStats()
        N.check(N.lib().ear_render_adjoint(self._h, C.byref(src), recs, len(recorders), C.byref(p),
                                           ptr, 1 if on_dev else 0, *ptrs, grad.ctypes.data,
                                           C.byref(st)))
        return grad, st.as_dict()

    def trace_debug(self, source: Source, recorders: Sequence[Recorder], *, band: int,
                    max_record: int, keyframe: int = -1, **kw):
        """Per-ray, per-reflection hit triangle (original index; -1 miss, -2
        path ended), bounce type and recorder-visibility mask."""
        src, _keep = source.at(keyframe)
        recs = recorders_at(recorders, keyframe)
        kw = dict(kw)
        kw["bands"] = (band,)
        p = make_params(**kw)
        n = int(p.num_rays)
        hit = np.empty((n, max_record), np.int32)
        bt = np.empty((n, max_record), np.uint8)
        vis = np.empty((n, max_record), np.uint32)
        N.check(N.lib().ear_trace_debug(self._h, C.byref(src), recs, len(recorders), C.byref(p),
                                        band, max_record, hit.ctypes.data, bt.ctypes.data,
                                        vis.ctypes.data))
        return hit, bt, vis

    def close(self):
        if getattr(self, "_h", None):
            N.lib().ear_scene_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Scene:
    """Mirror of the reference's Scene (src/Scene.h:42-79) over the GPU
    tracer.  Meshes are (n, 9) triangle arrays tagged with a material name."""

    def __init__(self, device: int = 0, box_pad: float = -1.0, visibility_map: int = 0):
        self.device = device
        self.box_pad = box_pad
        self.visibility_map = visibility_map
        self.meshes: list[tuple[np.ndarray, str]] = []
        self.materials: dict[str, Material] = {}
        self.listeners: list[Recorder] = []
        self.sources: list[Source] = []
        self._tracer: Optional[Tracer] = None

    # Scene::addMesh / addMaterial / addListener / addSoundSource
    def addMesh(self, triangles: np.ndarray, material: str) -> None:
        self.meshes.append((np.asarray(triangles, np.float32).reshape(-1, 9), material))
        self._tracer = None

    def addMaterial(self, m: Material) -> None:
        self.materials[m.name] = m
        self._tracer = None

    def addListener(self, r: Recorder) -> None:
        self.listeners.append(r)

    def addSoundSource(self, s: Source) -> None:
        self.sources.append(s)

    def geometry(self):
        names = list(self.materials)
        idx = {n: i for i, n in enumerate(names)}
        if self.meshes:
            v = np.concatenate([m for m, _ in self.meshes], 0)
            ids = np.concatenate([np.full(len(m), idx[name], np.int32) for m, name in self.meshes])
        else:
            v = np.zeros((0, 9), np.float32)
            ids = np.zeros(0, np.int32)
        return v, ids, [self.materials[n] for n in names]

    def tracer(self) -> Tracer:
        if self._tracer is None:
            v, ids, mats = self.geometry()
            self._tracer = Tracer(v, ids, mats, device=self.device, box_pad=self.box_pad,
                                  visibility_map=self.visibility_map)
        return self._tracer

    def Render(self, band: int, sound: int, absorbtion_factor: float, num_samples: int, dry: float,
               recorders: Sequence[Recorder], keyframeID: int = -1, *, seed: int = 0,
               num_bins: int = 3 * N.SAMPLE_RATE, max_bounces: int = N.EAR_REFERENCE_MAX_BOUNCES,
               cutoff: float = N.EAR_REFERENCE_CUTOFF, exact: bool = False) -> RenderResult:
        """Scene::Render (src/Scene.cpp:111-318) for one band: returns the
        (tracks, num_bins) impulse responses of ``recorders``."""
        air = [0.0, 0.0, 0.0]
        air[band] = 1.0 - float(absorbtion_factor)
        context = ((sound & 0xFFFF) << 16) | ((keyframeID + 1) & 0xFFFF)
        res = self.tracer().render(self.sources[sound], recorders, keyframe=keyframeID, seed=seed,
                                   context=context, bands=(band,), num_rays=num_samples,
                                   max_bounces=max_bounces, num_bins=num_bins, cutoff=cutoff,
                                   air_absorption=air, dry=dry, exact=exact)
        res.hist = res.hist[:, band, :]
        res.first_sample = res.first_sample[:, band]
        res.last_sample = res.last_sample[:, band]
        return res

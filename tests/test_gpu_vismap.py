"""Listener visibility maps (ear_bvh_opts.visibility_map).

A visibility test answered from the recorder's direction lists runs the
tree's own triangle test on every triangle whose padded box meets the
segment, so its answer is the tree traversal's: per-ray, per-reflection
visibility masks stay bit-exact against the oracle (exact kernels), and
maps on or off give identical debug records.
"""
import dataclasses
import os

import numpy as np
import pytest

import oracle
from ear_gb300 import Recorder, Tracer, scenes

pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))


def _crowded_room():
    """The small test room with five more pillars and seven more recorders,
    two of them within a millimetre of a surface (their boxes' direction
    ranges cover whole cube faces)."""
    w = scenes.small_test_room(n_side=6)
    extra = [w.vertices]
    for x, y, h in [(2.0, 1.0, 3.0), (5.0, 3.5, 2.0), (6.5, 2.0, 3.5), (2.5, 4.5, 1.2), (4.5, 5.0, 2.8)]:
        extra.append(scenes.box_triangles(0.4, 0.5, h) + np.tile(np.array([x, y, 0.0], np.float32), 3))
    v = np.concatenate(extra, 0).astype(np.float32)
    ids = (np.arange(v.shape[0]) % 3).astype(np.int32)
    recs = list(w.recorders)
    for loc in [(1.0, 1.0, 1.0), (7.0, 5.5, 3.0), (3.0, 3.0, 0.0005), (2.2, 1.25, 1.5),
                (4.0, 0.5, 2.0), (0.0005, 3.0, 1.0), (5.2, 3.75, 2.2)]:
        recs.append(Recorder(location=np.array(loc, np.float32)))
    return dataclasses.replace(w, vertices=v, material_ids=ids, recorders=recs, name="crowded-room")


def _debug(w, vmap, nrays, max_record, band, width=0):
    kw = dict(w.render, num_rays=nrays)
    with Tracer(w.vertices, w.material_ids, w.materials, device=0, visibility_map=vmap,
                width=width) as tr:
        return tr.trace_debug(w.source, w.recorders, band=band, max_record=max_record, exact=True, **kw)


@pytest.mark.parametrize("res", [8, 32, 256])
def test_visibility_bit_exact_against_oracle(res):
    w = _crowded_room()
    nrays, max_record, band = 1500, 60, 1
    hit, bt, vis = _debug(w, res, nrays, max_record, band)
    kw = dict(w.render, num_rays=nrays, bands=(band,))
    ref = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders,
                        threads=THREADS, debug_band=band, debug_rays=nrays,
                        debug_max_record=max_record, **kw)
    rh, rb, rv = ref["debug"]
    np.testing.assert_array_equal(hit, rh)
    np.testing.assert_array_equal(bt, rb)
    np.testing.assert_array_equal(vis, rv)
    # some recorders are seen and some hidden
    full = (1 << len(w.recorders)) - 1
    v = vis[hit >= 0] & full
    assert (v != 0).any() and (v != full).any()


@pytest.mark.parametrize("width", [2, 4])
def test_maps_on_and_off_identical(width):
    w = _crowded_room()
    off = _debug(w, -1, 3000, 60, 0, width=width)
    for res in (16, 64):
        on = _debug(w, res, 3000, 60, 0, width=width)
        for a, b in zip(off, on):
            np.testing.assert_array_equal(a, b)


def test_maps_on_a_20000_triangle_room():
    pytest.importorskip("scipy")
    rooms, render = scenes.sweep_rooms(num_rooms=1, pairs_per_room=4, keyframes=1,
                                       min_tris=20000, max_tris=20000, seed=8)
    r = rooms[0]
    kw = dict(render, num_rays=3000, num_bins=44100)
    got = []
    for vmap in (-1, 64, 141):
        with Tracer(r.vertices, r.material_ids, r.materials, visibility_map=vmap) as tr:
            got.append(tr.trace_debug(r.sources[0], r.listeners, band=2, max_record=80, exact=True,
                                      **kw))
    for other in got[1:]:
        for a, b in zip(got[0], other):
            np.testing.assert_array_equal(a, b)


def test_render_exact_with_maps():
    """Counters and energies of an exact render with maps match the oracle;
    the maps are read, and the statistics say so."""
    w = _crowded_room()
    kw = dict(w.render, num_rays=3000)
    with Tracer(w.vertices, w.material_ids, w.materials, visibility_map=48) as tr:
        res = tr.render(w.source, w.recorders, exact=True, **kw)
        res2 = tr.render(w.source, w.recorders, exact=True, **kw)
    ref = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders,
                        threads=THREADS, **kw)
    for key in ("rays", "segments", "shadow_queries", "contributions", "sampler_overflows"):
        assert res.stats[key] == ref["counters"][key], key
    np.testing.assert_array_equal(res.first_sample, ref["first_sample"])
    np.testing.assert_array_equal(res.last_sample, ref["last_sample"])
    e_gpu = (np.asarray(res.hist, np.float64) ** 2).sum(-1)
    e_ref = (np.asarray(ref["hist64"], np.float64) ** 2).sum(-1)
    rel = np.abs(e_gpu - e_ref) / np.maximum(e_ref, 1e-300)
    assert rel.max() < 1e-5
    assert res.stats["map_entries"] > 0
    assert res.stats["map_build_ms"] > 0.0
    # the second render reuses the maps
    assert res2.stats["map_build_ms"] == 0.0
    assert res2.stats["map_entries"] == res.stats["map_entries"]


def test_fast_render_with_maps():
    """Fast kernels: the maps change neither the paths nor, beyond the fast
    triangle test's own rounding, the contributions."""
    w = _crowded_room()
    kw = dict(w.render, num_rays=20000)
    out = {}
    for vmap in (-1, 32):
        with Tracer(w.vertices, w.material_ids, w.materials, visibility_map=vmap) as tr:
            out[vmap] = tr.render(w.source, w.recorders, **kw)
    a, b = out[-1].stats, out[32].stats
    assert a["segments"] == b["segments"]
    assert a["shadow_queries"] == b["shadow_queries"]
    assert abs(a["contributions"] - b["contributions"]) <= 1e-4 * a["contributions"]
    assert a["map_entries"] == 0 and b["map_entries"] > 0
    assert b["node_visits"] < a["node_visits"]


def test_automatic_setting_and_rebuild():
    """The automatic setting builds maps for renders of at least as many
    paths as triangles, with 4 sqrt(triangles) cells per face edge (a
    multiple of 64, at least 64), and lets shorter renders use them once
    built; a rebuilt tree or another recorder set rebuilds them."""
    w = _crowded_room()
    kw = dict(w.render, num_rays=500)
    short = dict(w.render, num_rays=100)  # 300 paths < 864 triangles
    with Tracer(w.vertices, w.material_ids, w.materials) as tr:
        rs = tr.render(w.source, w.recorders, **short)
        assert rs.stats["map_entries"] == 0 and rs.stats["map_res"] == 0
        r0 = tr.render(w.source, w.recorders, **kw)
        assert r0.stats["map_entries"] > 0 and r0.stats["map_res"] == 64
        assert r0.stats["map_bytes"] > 0 and r0.stats["map_build_ms"] > 0
        rs = tr.render(w.source, w.recorders, **short)
        assert rs.stats["map_entries"] > 0 and rs.stats["map_build_ms"] == 0
        tr.build_bvh(visibility_map=24)
        r1 = tr.render(w.source, w.recorders, **kw)
        assert r1.stats["map_build_ms"] > 0 and r1.stats["map_entries"] > 0
        r2 = tr.render(w.source, w.recorders[:3], **kw)
        assert r2.stats["map_build_ms"] > 0
        tr.build_bvh(visibility_map=-1)
        assert tr.render(w.source, w.recorders, **kw).stats["map_entries"] == 0


def test_batch_with_maps_equals_plain_renders_without():
    """A batch builds one map per scene over its jobs' distinct recorder
    locations; its exact jobs count and record what plain renders without
    maps do."""
    from ear_gb300.batch import Batch, Job

    w = _crowded_room()
    render = dict(w.render, num_bins=44100)
    src = np.asarray(w.source.location, np.float32)
    sets = [w.recorders[:3], w.recorders[3:6], [w.recorders[6], w.recorders[0]], w.recorders[7:]]
    jobs = [Job(scene=0, source=type(w.source)(location=src + np.float32(0.3 * k), gain=0.8),
                recorders=rs, num_rays=700 + 100 * k, context=k) for k, rs in enumerate(sets)]
    with Tracer(w.vertices, w.material_ids, w.materials, visibility_map=40) as on, \
            Tracer(w.vertices, w.material_ids, w.materials, visibility_map=-1) as off:
        plain = [off.render(j.source, j.recorders, exact=True,
                            **dict(render, num_rays=j.num_rays, context=j.context)) for j in jobs]
        b = Batch([on], jobs, exact=True, **{k: v for k, v in render.items() if k != "num_rays"})
        st = b.run()
        assert st["map_bytes"] > 0 and st["map_res"] == 40 and st["map_entries"] > 0
        for k in ("segments", "shadow_queries", "contributions", "rays"):
            assert int(st[k]) == sum(int(p.stats[k]) for p in plain), k
        for i, p in enumerate(plain):
            r = b.result(i)
            np.testing.assert_array_equal(r.first_sample, p.first_sample)
            np.testing.assert_array_equal(r.last_sample, p.last_sample)
            e1 = (np.asarray(r.hist, np.float64) ** 2).sum(-1)
            e2 = (np.asarray(p.hist, np.float64) ** 2).sum(-1)
            assert (np.abs(e1 - e2) <= 1e-5 * np.maximum(e2, 1e-30)).all(), i
        b.close()


def _grazing_room():
    """A 20 x 20 x 4 m box of 12 large triangles (and a 5 cm step) whose
    recorders sit 0.1 to 2 mm above the floor and 0.1 mm from a wall: the
    segments from path
    vertices on the floor and that wall to them graze the large triangles'
    planes (cosines down to about 1e-5), where the triangle test's own
    rounding decides near-zero crossings."""
    w = scenes.shoebox()
    # the room and a 5 cm step on its floor (occludes some grazing segments)
    step = scenes.box_triangles(4.0, 3.0, 0.05) + np.tile(np.array([6.0, 8.0, 0.0], np.float32), 3)
    v = np.concatenate([scenes.box_triangles(20.0, 20.0, 4.0), step], 0).astype(np.float32)
    recs = [Recorder(location=np.array(p, np.float32)) for p in
            [(10.0, 10.0, 0.0001), (3.0, 15.0, 0.0005), (17.0, 4.0, 0.002), (0.0001, 10.0, 1.5),
             (15.0, 15.0, 0.0001)]]
    return dataclasses.replace(w, vertices=v, material_ids=np.zeros(len(v), np.int32),
                               recorders=recs, name="grazing-box",
                               render=dict(w.render, num_bins=88200))


def test_grazing_segments_bit_exact_maps_on_off_and_oracle():
    w = _grazing_room()
    nrays, max_record, band = 3000, 40, 1
    off = _debug(w, -1, nrays, max_record, band)
    kw = dict(w.render, num_rays=nrays, bands=(band,))
    ref = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders,
                        threads=THREADS, debug_band=band, debug_rays=nrays,
                        debug_max_record=max_record, **kw)
    for a, b in zip(off, ref["debug"]):
        np.testing.assert_array_equal(a, b)
    for res in (8, 64, 256):
        on = _debug(w, res, nrays, max_record, band)
        for a, b in zip(off, on):
            np.testing.assert_array_equal(a, b)
    # the floor's recorders are seen from some vertices and hidden from others
    full = (1 << len(w.recorders)) - 1
    vis = off[2][off[0] >= 0] & full
    assert (vis != 0).any() and (vis != full).any()

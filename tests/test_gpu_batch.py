"""Batched rendering (ear_batch_*): every job of a batch renders what
ear_render renders for the same scene, source, recorders, seed and context
-- the same rays (exact kernels: identical counters and bookkeeping) and
the same histograms up to float-atomic ordering -- through graph replays,
source moves, schedule changes and the autotuner (including BVH leaf
sizes, which change no result)."""
import numpy as np
import pytest

pytest.importorskip("scipy")
from ear_gb300 import Tracer, scenes  # noqa: E402
from ear_gb300.batch import Batch, Job  # noqa: E402

pytestmark = pytest.mark.gpu
KEYS = ("segments", "shadow_queries", "contributions", "rays")


@pytest.fixture(scope="module")
def sweep():
    rooms, render = scenes.sweep_rooms(num_rooms=3, pairs_per_room=2, keyframes=3,
                                       min_tris=300, max_tris=6000, seed=5)
    render = dict(render, num_rays=1500, num_bins=44100)
    tracers = [Tracer(r.vertices, r.material_ids, r.materials) for r in rooms]
    jobs = []
    for ri, r in enumerate(rooms):
        for pi, (s, l) in enumerate(zip(r.sources, r.listeners)):
            for k in range(3):
                jobs.append(Job(scene=ri, source=s, recorders=[l], keyframe=k,
                                num_rays=1000 + 250 * k, context=100 * ri + 10 * pi + k))
    yield rooms, render, tracers, jobs
    for t in tracers:
        t.close()


def _plain(tracers, jobs, render, exact=True):
    out = []
    for j in jobs:
        kw = dict(render, num_rays=j.num_rays, context=j.context)
        out.append(tracers[j.scene].render(j.source, j.recorders, keyframe=j.keyframe,
                                           exact=exact, **kw))
    return out


def _energy(h):
    return (np.asarray(h, np.float64) ** 2).sum(-1)


def _check(batch, plain, stats):
    tot = {k: sum(int(p.stats[k]) for p in plain) for k in KEYS}
    for k in KEYS:
        assert int(stats[k]) == tot[k], k
    for i, p in enumerate(plain):
        r = batch.result(i)
        np.testing.assert_array_equal(r.first_sample, p.first_sample)
        np.testing.assert_array_equal(r.last_sample, p.last_sample)
        e1, e2 = _energy(r.hist), _energy(p.hist)
        assert (np.abs(e1 - e2) <= 1e-5 * np.maximum(e2, 1e-30)).all(), i


def test_batch_equals_plain_renders(sweep):
    rooms, render, tracers, jobs = sweep
    plain = _plain(tracers, jobs, render)
    with Batch(tracers, jobs, exact=True, **{k: v for k, v in render.items() if k != "num_rays"}) as b:
        st = b.run()
        _check(b, plain, st)
        # graph replay: same rays again
        st2 = b.run()
        for k in KEYS:
            assert st2[k] == st[k]
        _check(b, plain, st2)
        # without the graph, and with another schedule
        b.set_config(block=128, blocks_per_sm=3, no_graph=True)
        _check(b, plain, b.run())


def test_batch_set_sources_moves_every_job(sweep):
    rooms, render, tracers, jobs = sweep
    moved = [Job(scene=j.scene, source=j.source, recorders=j.recorders,
                 keyframe=min(j.keyframe + 1, 2), num_rays=j.num_rays, context=j.context)
             for j in jobs]
    pos = np.stack([j.source.location[j.keyframe] for j in moved])
    kw = {k: v for k, v in render.items() if k != "num_rays"}
    with Batch(tracers, jobs, exact=True, **kw) as b:
        b.run()
        b.set_sources(pos)
        st = b.run()
    _check_after = _plain(tracers, moved, render)
    tot = sum(int(p.stats["segments"]) for p in _check_after)
    assert int(st["segments"]) == tot


def test_autotuner_applies_a_schedule_and_changes_no_result(sweep, tmp_path):
    rooms, render, tracers, jobs = sweep
    plain = _plain(tracers, jobs, render)
    kw = {k: v for k, v in render.items() if k != "num_rays"}
    cache = tmp_path / "tune.txt"
    for t in tracers:  # leaf sizes apply to LBVH scenes
        t.build_bvh(builder="lbvh")
    with Batch(tracers, jobs, exact=True, **kw) as b:
        res = b.tune(trial_fraction=0.5, tune_leaf_size=True, repeats=1, cache_path=str(cache),
                     tune_width=True)
        assert res["candidates"] >= 8 and not res["from_cache"]
        assert res["best_ms"] > 0 and res["default_ms"] > 0
        cfg = b.config
        assert cfg["max_leaf_size"] in (1, 2, 4) and cfg["block"] in (128, 256)
        assert cfg["bvh_width"] in (2, 4)
        _check(b, plain, b.run())
    # a second batch of the same shape takes the cached schedule
    with Batch(tracers, jobs, exact=True, **kw) as b:
        res2 = b.tune(tune_leaf_size=True, cache_path=str(cache), tune_width=True)
        assert res2["from_cache"] and res2["best"]["block"] == res["best"]["block"]
        assert res2["best"]["bvh_width"] == res["best"]["bvh_width"]
        _check(b, plain, b.run())
    for t in tracers:  # back to the default builder and width for the other tests
        t.build_bvh()


def test_leaf_size_changes_no_hit(sweep):
    """Closest hits and visibility are independent of the BVH leaf size."""
    import ctypes as C
    from ear_gb300 import _native as N
    rooms, render, tracers, jobs = sweep
    r = rooms[-1]
    kw = dict(render, num_rays=400, context=3)
    with Tracer(r.vertices, r.material_ids, r.materials, builder="lbvh") as t:
        ref = t.trace_debug(r.sources[0], r.listeners[:1], band=1, max_record=60, keyframe=0,
                            exact=True, **kw)
        for leaf in (2, 4, 16):
            o = N.EarBvhOpts()
            o.box_pad = -1.0
            o.max_leaf_size = leaf
            o.builder = N.EAR_BVH_LBVH
            N.check(N.lib().ear_scene_build_bvh(t._h, C.byref(o)))
            got = t.trace_debug(r.sources[0], r.listeners[:1], band=1, max_record=60,
                                keyframe=0, exact=True, **kw)
            for a, b in zip(ref, got):
                np.testing.assert_array_equal(a, b)


def test_one_shot_render_batch(sweep):
    import ctypes as C
    from ear_gb300 import _native as N
    from ear_gb300.scene import make_params
    rooms, render, tracers, jobs = sweep
    js = jobs[:4]
    plain = _plain(tracers, js, render)
    scenes_arr = (C.c_void_p * len(tracers))(*[t._h.value for t in tracers])
    cj = (N.EarBatchJob * len(js))()
    keep = []
    for i, j in enumerate(js):
        rec = (N.EarRecorder * 1)(j.recorders[0].at(j.keyframe))
        keep.append(rec)
        cj[i].scene, cj[i].num_recorders, cj[i].recorders = j.scene, 1, rec
        cj[i].source[:] = list(j.source.location[j.keyframe])
        cj[i].gain, cj[i].num_rays, cj[i].context = 1.0, j.num_rays, j.context
    p = make_params(exact=True, **{k: v for k, v in render.items() if k != "num_rays"})
    outs = (N.EarHistograms * len(js))()
    hs = []
    for i in range(len(js)):
        h = np.zeros((1, 3, render["num_bins"]), np.float32)
        f = np.zeros((1, 3), np.int32)
        l = np.zeros((1, 3), np.int32)
        hs.append((h, f, l))
        outs[i].data, outs[i].first_sample, outs[i].last_sample = h.ctypes.data, f.ctypes.data, l.ctypes.data
    st = N.EarRenderStats()
    N.check(N.lib().ear_render_batch(scenes_arr, len(tracers), cj, len(js), C.byref(p), outs,
                                     C.byref(st)))
    assert st.segments == sum(int(q.stats["segments"]) for q in plain)
    for (h, f, l), q in zip(hs, plain):
        np.testing.assert_array_equal(f, q.first_sample)
        np.testing.assert_array_equal(l, q.last_sample)
        e1, e2 = _energy(h), _energy(q.hist)
        assert (np.abs(e1 - e2) <= 1e-5 * np.maximum(e2, 1e-30)).all()

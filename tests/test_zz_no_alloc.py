"""ear_render_noalloc: the render entry point for callers that must not
allocate (an audio engine re-rendering from its real-time thread, a host
holding the tracer to a fixed GPU memory budget).  It is called through the
C ABI twice in a row and must match ear_render; it must also reject
requests beyond its fixed scratch.  Collected last on purpose: if it fails,
a run that stops at the first failure has already run every other test."""
import ctypes as C

import numpy as np
import pytest

from ear_gb300 import Source, Tracer, _native as N, scenes
from ear_gb300.scene import make_params, recorders_at

pytestmark = pytest.mark.gpu


def _energy(h):
    return (np.asarray(h, np.float64) ** 2).sum(-1)


def _noalloc(tr, w, params, out):
    src, _keep = w.source.at(-1)
    recs = recorders_at(w.recorders, -1)
    tracks = w.num_tracks
    first = np.zeros((tracks, 3), np.int32)
    last = np.zeros((tracks, 3), np.int32)
    st = N.EarRenderStats()
    rc = N.lib().ear_render_noalloc(tr._h, C.byref(src), recs, len(w.recorders), C.byref(params),
                                    out.data_ptr(), first.ctypes.data, last.ctypes.data,
                                    C.byref(st))
    return rc, first, last, st.as_dict()


@pytest.mark.parametrize("exact", [True, False])
def test_noalloc_matches_render_twice(exact):
    torch = pytest.importorskip("torch")
    w = scenes.small_test_room()
    kw = dict(w.render)
    kw["num_rays"] = 3000
    with Tracer(w.vertices, w.material_ids, w.materials, device=0) as tr:
        ref = tr.render(w.source, w.recorders, exact=exact, **kw)
        params = make_params(exact=exact, **kw)
        out = torch.empty((w.num_tracks, 3, kw["num_bins"]), dtype=torch.float32, device="cuda")
        for call in range(2):
            out.fill_(123.0)  # the call must zero the buffer itself
            torch.cuda.synchronize()
            free0 = torch.cuda.mem_get_info()[0]
            rc, first, last, stats = _noalloc(tr, w, params, out)
            torch.cuda.synchronize()
            assert rc == N.EAR_OK, N.lib().ear_last_error()
            if call:
                # the defining property: once the first call has resolved
                # the scratch address, a call takes no device memory
                assert torch.cuda.mem_get_info()[0] == free0
            got = out.cpu().numpy()
            e_got, e_ref = _energy(got), _energy(ref.hist)
            assert (np.abs(e_got - e_ref) <= 1e-5 * np.maximum(e_ref, 1e-300)).all()
            scale = np.abs(ref.hist).max()
            assert np.abs(got - ref.hist).max() <= 1e-5 * scale
            np.testing.assert_array_equal(first, ref.first_sample)
            np.testing.assert_array_equal(last, ref.last_sample)
            for key in ("rays", "segments", "shadow_queries", "contributions"):
                assert stats[key] == ref.stats[key], key
            # the visibility maps ear_render built are read, not rebuilt
            assert stats["map_res"] == ref.stats["map_res"] > 0
            assert stats["map_entries"] == ref.stats["map_entries"]
            assert stats["map_build_ms"] == 0.0


def test_noalloc_without_maps_traverses_the_tree():
    """With no map built for the recorder set, the no-alloc render builds
    none and matches ear_render without maps."""
    torch = pytest.importorskip("torch")
    w = scenes.small_test_room()
    kw = dict(w.render)
    kw["num_rays"] = 2000
    with Tracer(w.vertices, w.material_ids, w.materials, device=0, visibility_map=-1) as tr:
        ref = tr.render(w.source, w.recorders, exact=True, **kw)
        params = make_params(exact=True, **kw)
        out = torch.empty((w.num_tracks, 3, kw["num_bins"]), dtype=torch.float32, device="cuda")
        rc, first, last, stats = _noalloc(tr, w, params, out)
        assert rc == N.EAR_OK, N.lib().ear_last_error()
        assert stats["map_entries"] == 0 and stats["map_res"] == 0
        for key in ("rays", "segments", "shadow_queries", "contributions"):
            assert stats[key] == ref.stats[key], key
        np.testing.assert_array_equal(first, ref.first_sample)


def test_noalloc_rejects_requests_beyond_its_scratch():
    torch = pytest.importorskip("torch")
    w = scenes.small_test_room()
    kw = dict(w.render)
    kw["num_rays"] = 10
    with Tracer(w.vertices, w.material_ids, w.materials, device=0) as tr:
        out = torch.full((2 * 33, 3, kw["num_bins"]), 7.0, dtype=torch.float32, device="cuda")
        params = make_params(**kw)
        src, _ = w.source.at(-1)
        many = recorders_at(w.recorders * 17, -1)  # 34 recorders
        rc = N.lib().ear_render_noalloc(tr._h, C.byref(src), many, 34, C.byref(params),
                                        out.data_ptr(), None, None, None)
        assert rc == N.EAR_ERR_INVALID_ARG and b"at most 32" in N.lib().ear_last_error()
        emitter = Source(emitter=np.array([[2, 2, 1, 2.5, 2, 1, 2, 2.5, 1.2]], np.float32))
        esrc, _keep = emitter.at(-1)
        recs = recorders_at(w.recorders, -1)
        rc = N.lib().ear_render_noalloc(tr._h, C.byref(esrc), recs, 2, C.byref(params),
                                        out.data_ptr(), None, None, None)
        assert rc == N.EAR_ERR_UNSUPPORTED
        odd = make_params(**dict(kw, num_bins=kw["num_bins"] + 1))
        rc = N.lib().ear_render_noalloc(tr._h, C.byref(src), recs, 2, C.byref(odd),
                                        out.data_ptr(), None, None, None)
        assert rc == N.EAR_ERR_INVALID_ARG and b"multiple of 4" in N.lib().ear_last_error()
        # rejected calls queue no device work: the caller's buffer is as it was
        assert bool((out == 7.0).all())

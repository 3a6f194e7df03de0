"""The oracle pinned to the reference itself: the reference's own
Scene::Render (src/Scene.cpp:111-318), its parsers, materials and
recorders, compiled from its sources into oracle/_ref by
oracle/build_ref.py (against a GMTL / Boost interface shim), renders the
same .EAR scene on the oracle's random numbers.  Its FloatBuffer tracks
must equal the oracle's float accumulation bit for bit, with the same
first_sample / real_length bookkeeping and the same number of random draws.

Where the reference tree is absent (the GPU machine), the live comparison
skips and the committed fixture of the reference's output
(tests/golden/reference_render.json, made by
tests/golden/make_reference_golden.py) pins the oracle instead."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import oracle
from ear_gb300 import scenes

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden" / "reference_render.json"


def _ref_lib():
    import importlib.util

    spec = importlib.util.spec_from_file_location("build_ref", ROOT / "oracle" / "build_ref.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    if mod.build_render() is None:
        pytest.skip("the reference tree is not present (oracle/_ref cannot be built)")


def _relief_small():
    w = scenes.relief_hall()
    return w


CASES = {
    # stereo + mono, refraction, an always-reflecting band, air absorption, gain
    "small_test_room": (scenes.small_test_room, 2000, 44100),
    # the configs' 12-triangle specular shoebox
    "shoebox": (scenes.shoebox, 2000, 88200),
    # 8 materials with refraction (the inverse problem's scene)
    "inverse_shoebox": (lambda: scenes.inverse_shoebox(num_rays=1)[0], 1000, 88200),
    # 20,000 displaced triangles, 8 materials, stereo (at least 50 rays: the
    # reference's progress bar divides by num_samples / 50, src/HelperFunctions.cpp:62-63)
    "relief_hall": (_relief_small, 60, 132300),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_reference_render_equals_oracle(name, tmp_path):
    _ref_lib()
    make, rays, window = CASES[name]
    w = make()
    ref = oracle.reference_render(w, tmp_path, rays, window)
    V, M = oracle.grouped_by_material(w)
    kw = oracle.reference_pin_params(w, rays, window)
    for b in range(3):
        # every uniform of the tape is drawn, none more: the reference makes
        # the same random decisions in the same order
        assert ref["used"][b] == ref["tape"][b] > 0
        o = oracle.render(V, M, w.materials, w.source, w.recorders, threads=1,
                          **dict(kw, bands=(b,)))
        got = o["hist32"][:, b]
        np.testing.assert_array_equal(ref["tracks"][:, b].view(np.uint32), got.view(np.uint32))
        np.testing.assert_array_equal(ref["first_sample"][:, b], o["first_sample"][:, b])
        np.testing.assert_array_equal(np.minimum(ref["real_length"][:, b], window),
                                      o["last_sample"][:, b])
        assert np.abs(got).max() > 0


def _track_digest(x):
    return hashlib.sha256(np.ascontiguousarray(x, np.float32).tobytes()).hexdigest()


def test_oracle_equals_reference_fixture():
    """Runs everywhere: the oracle reproduces, bit for bit, the tracks the
    reference's own render produced when the fixture was made."""
    g = json.loads(GOLDEN.read_text())
    for case in g["cases"]:
        make, _, _ = CASES[case["name"]]
        w = make()
        rays, window = case["rays"], case["window"]
        V, M = oracle.grouped_by_material(w)
        kw = oracle.reference_pin_params(w, rays, window)
        for b in range(3):
            o = oracle.render(V, M, w.materials, w.source, w.recorders, threads=1,
                              **dict(kw, bands=(b,)))
            for t in range(len(case["tracks"])):
                ref = case["tracks"][t][b]
                assert _track_digest(o["hist32"][t, b]) == ref["sha256"], (case["name"], t, b)
                assert int(o["first_sample"][t, b]) == ref["first_sample"]
                assert int(o["last_sample"][t, b]) == min(ref["real_length"], window)


T60_CASES = {
    # name: (workload, samples in the settings block (samples / 10 rays), window)
    "shoebox": (scenes.shoebox, 600, 88200),
    "small_test_room": (scenes.small_test_room, 600, 44100),
}


def _calc_t60_from_oracle(w, rays, window):
    """`EAR calc T60` from this library's post-processing and statistics
    (the calls the command line makes) on the oracle's mid-band render."""
    import ctypes as C

    from ear_gb300 import _native as N, post

    V, M = oracle.grouped_by_material(w)
    kw = oracle.reference_pin_params(w, rays, window)
    o = oracle.render(V, M, w.materials, w.source, w.recorders, threads=1,
                      **dict(kw, bands=(1,)))
    t_ear = post.calc_t60(o["hist32"][:, 1], o["first_sample"][:, 1], o["last_sample"][:, 1],
                          tracks_per_recorder=[r.tracks for r in w.recorders])
    ids, counts = np.unique(M, return_counts=True)  # one MESH block per material
    blocks = counts.astype(np.int64)
    mat = w.materials[int(ids[0])].to_c()
    stats = np.zeros(5, np.float32)
    air_mid = float(np.float32(w.render.get("air_absorption", (0.0, 0.0, 0.0))[1]))
    N.check(N.lib().ear_statistical_t60(np.ascontiguousarray(V, np.float32).ctypes.data,
                                        blocks.ctypes.data, len(blocks), C.byref(mat), air_mid,
                                        stats.ctypes.data))
    return np.array([t_ear, stats[3], stats[4]], np.float32)


@pytest.mark.parametrize("name", sorted(T60_CASES))
def test_reference_calc_t60_equals_library(name, tmp_path):
    """The reference's `EAR calc T60` branch (src/EAR.cpp:55-284) -- its
    render, Recorder::Power / Truncate, RecorderTrack::T60 and the Sabine /
    Norris-Eyring formulas on Mesh::Volume / Area / TotalAbsorption /
    AverageAbsorption -- gives the same three floats, bit for bit, as this
    library's post-processing and statistics on the oracle's render."""
    _ref_lib()
    make, samples, window = T60_CASES[name]
    w = make()
    ref = oracle.reference_calc_t60(w, tmp_path, samples, window)
    assert ref["num_rays"] == samples // 10
    assert ref["used"] == ref["tape"] > 0
    ours = _calc_t60_from_oracle(w, samples // 10, window)
    assert ref["t60"][0] > 0 and ref["t60"][1] > 0 and ref["t60"][2] > 0
    np.testing.assert_array_equal(ref["t60"].view(np.uint32), ours.view(np.uint32))


def test_library_calc_t60_equals_reference_fixture():
    """Runs everywhere: the library's post-processing and statistics on the
    oracle's render give the reference's `EAR calc T60` floats recorded in
    the fixture, bit for bit."""
    g = json.loads(GOLDEN.read_text())
    assert {c["name"] for c in g["calc_t60"]} == set(T60_CASES)
    for case in g["calc_t60"]:
        make, _, _ = T60_CASES[case["name"]]
        ours = _calc_t60_from_oracle(make(), case["samples"] // 10, case["window"])
        assert ours.view(np.uint32).tolist() == case["t60_bits"], case["name"]

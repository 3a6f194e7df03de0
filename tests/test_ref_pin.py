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

"""The .EAR scene format (Python writer/reader and the C++ reader/writer of
the EAR command line) and the golden fixtures of tests/golden/."""
import ctypes as C
import hashlib
import json
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle
from ear_gb300 import Material, earfile, scenes

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = ROOT / "tests" / "golden"
CLI = ROOT / "ear_gb300" / "bin" / "EAR"


def cli(*args):
    return subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=60)


def test_presets_fixture_matches_reference_formulas():
    """The presets read from the reference add-on derive, in the oracle, to
    the survival / reflection probabilities of src/Material.cpp."""
    pre = json.loads((GOLDEN / "material_presets.json").read_text())
    assert [p["name"] for p in pre] == ["100% Transparent", "100% Absorbent", "100% Reflecting",
                                       "Rough concrete", "Smooth concrete", "Wooden floor", "Glazing"]
    for p in pre:
        m = Material(reflection=p["refl"], refraction=p["refr"], specularity=p["spec"])
        surv = (C.c_float * 3)()
        prob = (C.c_float * 3)()
        alw = (C.c_int32 * 3)()
        spec = (C.c_float * 3)()
        assert oracle.lib().oracle_material(C.byref(m.to_c()), surv, prob, alw, spec) == 0
        for b, d in enumerate(p["derived"]):
            assert surv[b] == pytest.approx(d["survival"], abs=0.0), p["name"]
            assert bool(alw[b]) == d["always_reflect"]
            if d["p_reflect"] is not None:
                assert prob[b] == d["p_reflect"]


def test_python_reader_reads_presets_room():
    sc = earfile.read_ear(GOLDEN / "presets_room.ear")
    pre = json.loads((GOLDEN / "material_presets.json").read_text())
    assert [m[0] for m in sc.materials] == [p["name"] for p in pre[1:7]]
    assert sum(len(t) for _, t in sc.meshes) == 12
    assert sc.settings["samples"] == 10000
    assert [r["channels"] for r in sc.recorders] == [1, 2]
    np.testing.assert_allclose(sc.recorders[1]["right_ear"], [0, -1, 0])


def test_cli_reader_and_writer_round_trip(tmp_path):
    r = cli("info", GOLDEN / "presets_room.ear", "--resave", tmp_path / "again.ear")
    assert r.returncode == 0, r.stdout
    info = json.loads(r.stdout.strip().splitlines()[-1])
    assert info == {"materials": 6, "meshes": 6, "triangles": 12, "recorders": 2, "stereo": 1,
                    "sources": 1, "keys": 0, "settings": 5, "unknown": 0}
    assert (tmp_path / "again.ear").read_bytes() == (GOLDEN / "presets_room.ear").read_bytes()


def test_python_and_cli_agree_on_a_generated_scene(tmp_path):
    w = scenes.small_test_room()
    b = earfile.workload_to_ear(w, samples=12345, keys=None)
    p = tmp_path / "room.ear"
    p.write_bytes(b)
    r = cli("info", p, "--resave", tmp_path / "room2.ear")
    assert r.returncode == 0, r.stdout
    assert (tmp_path / "room2.ear").read_bytes() == b
    info = json.loads(r.stdout.strip().splitlines()[-1])
    assert info["triangles"] == w.num_triangles and info["recorders"] == 2


def test_animated_blocks_and_unknown_blocks(tmp_path):
    keys = [0.0, 0.5, 1.0]
    b = earfile.encode(
        materials=[("m", (0.8, 0.8, 0.8), (0.0, 0.0, 0.0), (0.1, 0.1, 0.1))],
        meshes=[("m", scenes.box_triangles(4, 4, 3))],
        sources=[{"location": [[1, 1, 1], [1.5, 1, 1], [2, 1, 1]]}],
        recorders=[{"location": [[3, 3, 1.5]] * 3, "channels": 2,
                    "right_ear": [[0, -1, 0], [0, -1, 0], [1, 0, 0]]}],
        keys=keys)
    # append an unknown block and a lowercase mesh-emitter block, which the
    # reference does not recognise and skips (src/EAR.cpp:115-118)
    b += b"XTRA" + (4).to_bytes(4, "little") + b"abcd"
    b += earfile._block("ssrc", ["e.wav", 1.0])
    p = tmp_path / "anim.ear"
    p.write_bytes(b)
    sc = earfile.read_ear(p)
    assert sc.keys == keys and sc.sources[0]["location"].shape == (3, 3)
    assert sc.unknown == ["XTRA", "ssrc"]
    r = cli("info", p)
    assert r.returncode == 0
    info = json.loads(r.stdout.strip().splitlines()[-1])
    assert info["keys"] == 3 and info["unknown"] == 2


def test_truncated_and_foreign_files_are_errors(tmp_path):
    good = (GOLDEN / "presets_room.ear").read_bytes()
    (tmp_path / "cut.ear").write_bytes(good[:-7])
    r = cli("info", tmp_path / "cut.ear")
    assert r.returncode == 1 and "Error" in r.stdout
    (tmp_path / "x.ear").write_bytes(b"RIFF....")
    r = cli("info", tmp_path / "x.ear")
    assert r.returncode == 1 and "Failed to read file" in r.stdout
    r = cli("calc", "T60", tmp_path / "x.ear")
    assert r.returncode == 1
    assert cli("test").returncode == 0


def test_oracle_golden_shoebox():
    """The oracle still reproduces its committed shoebox outputs."""
    g = json.loads((GOLDEN / "oracle_shoebox.json").read_text())
    w = scenes.shoebox()
    kw = dict(w.render)
    kw["num_rays"] = g["config"]["rays_per_band"]
    r = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders, threads=3,
                      debug_band=1, debug_rays=kw["num_rays"], debug_max_record=50, **kw)
    hit, _bt, vis = r["debug"]
    assert r["counters"] == g["counters"]
    assert hashlib.sha256(hit.tobytes()).hexdigest() == g["hits_sha256"]
    assert hashlib.sha256(vis.tobytes()).hexdigest() == g["visible_sha256"]
    np.testing.assert_allclose((r["hist64"] ** 2).sum(-1), g["energy"], rtol=1e-12)
    assert r["first_sample"].tolist() == g["first_sample"]
    assert r["last_sample"].tolist() == g["last_sample"]

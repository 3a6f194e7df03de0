"""Generates tests/golden/reference_render.json: the output of the
reference's own Scene::Render (oracle/_ref/libear_ref_render.so, built by
oracle/build_ref.py from the reference tree) on the scenes of
tests/test_ref_pin.py, per (track, band): first_sample, real_length, a
SHA-256 of the float32 track over the window, its energy and the energy
of 64 equal time blocks.  The oracle must reproduce the digests bit for
bit (tests/test_ref_pin.py) and the GPU's exact kernels the energies
within 1e-5 (tests/test_gpu_parity.py), where the reference tree is
absent.  It also holds the reference's `EAR calc T60` results (T60 from
the rendered response, Sabine, Norris-Eyring) on the scenes of
test_ref_pin.T60_CASES, as float32 bit patterns.

    python tests/golden/make_reference_golden.py [--reference REFERENCE_ROOT]

REFERENCE_ROOT defaults to $EAR_REFERENCE_ROOT, else to a checkout named
``reference`` beside this repository.
"""
from __future__ import annotations

import argparse
import hashlib
import json
import os
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

# (case, rays per band, window in samples): small enough for a fixture,
# large enough to exercise every branch of the bounce body
FIXTURE = [("small_test_room", 300, 44100), ("shoebox", 300, 88200)]


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=None)
    args = ap.parse_args()
    if args.reference:
        os.environ["EAR_REFERENCE_ROOT"] = args.reference
    import importlib.util

    spec = importlib.util.spec_from_file_location("build_ref", ROOT / "oracle" / "build_ref.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    from ear_gb300.build import build_oracle

    build_oracle()
    if mod.build_render() is None:
        sys.exit("the reference tree is not present")
    import oracle

    sys.path.insert(0, str(ROOT / "tests"))
    from test_ref_pin import CASES, T60_CASES

    cases = []
    for name, rays, window in FIXTURE:
        w = CASES[name][0]()
        with tempfile.TemporaryDirectory() as d:
            r = oracle.reference_render(w, d, rays, window)
        tracks = []
        for t in range(r["tracks"].shape[0]):
            row = []
            for b in range(3):
                x = r["tracks"][t, b]
                e = x.astype(np.float64) ** 2
                row.append({"first_sample": int(r["first_sample"][t, b]),
                            "real_length": int(r["real_length"][t, b]),
                            "sha256": hashlib.sha256(x.tobytes()).hexdigest(),
                            "energy": float(e.sum()),
                            "block_energy": [float(c.sum()) for c in np.array_split(e, 64)]})
            tracks.append(row)
        cases.append({"name": name, "rays": rays, "window": window, "tape": r["tape"],
                      "tracks": tracks})
    t60 = []
    for name in sorted(T60_CASES):
        make, samples, window = T60_CASES[name]
        with tempfile.TemporaryDirectory() as d:
            r = oracle.reference_calc_t60(make(), d, samples, window)
        t60.append({"name": name, "samples": samples, "window": window,
                    "t60_bits": [int(x) for x in r["t60"].view(np.uint32)],
                    "t60": [float(x) for x in r["t60"]]})
    out = {"what": "the reference's own Scene::Render (src/Scene.cpp:111-318) compiled from its "
                   "sources with a GMTL/Boost interface shim, on the oracle's random tape; "
                   "max 1000 path vertices, cut-off 1e-8, point source, static",
           "cases": cases,
           "calc_t60_what": "the `EAR calc T60` branch of src/EAR.cpp:55-284 on the same build: "
                            "(T60_ear, T60_sabine, T60_eyring)",
           "calc_t60": t60}
    (HERE / "reference_render.json").write_text(json.dumps(out, indent=1))
    print("wrote", HERE / "reference_render.json")


if __name__ == "__main__":
    main()

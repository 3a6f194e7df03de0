"""Generates the golden fixtures in this directory.

    python tests/golden/make_golden.py [--reference REFERENCE_ROOT]

REFERENCE_ROOT defaults to $EAR_REFERENCE_ROOT, else to a checkout named
``reference`` beside this repository.

* material_presets.json -- the 7 material presets of the reference's Blender
  add-on, read by importing blender/render_EAR/materials.py from the
  reference checkout (plain Python, no Blender needed): name and the
  refl/refr/spec triplets the exporter writes into MAT blocks
  (blender/render_EAR/__init__.py:206-208), plus the derived per-band
  survival (Material::absorption_coefficient, src/Material.cpp:33-60) and
  reflection probability (Material::Bounce, src/Material.cpp:76-83)
  computed here with float32 arithmetic in the reference's order.
* presets_room.ear -- a 5x4x3 m room whose six walls use the six non-custom
  presets, written in the exporter's encoding (ear_gb300.earfile).
* oracle_shoebox.json -- the oracle's path counters, per-band energies and
  a checksum of per-bounce hit indices for a small seeded shoebox render:
  pins the CPU restatement against accidental change.
"""
from __future__ import annotations

import argparse
import hashlib
import importlib.util
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)


def f32(x):
    return np.float32(x)


def derive(refl, refr):
    """Material::Material / Material::Bounce in float32, reference order."""
    out = []
    for b in range(3):
        a = f32(1.0)
        a = f32(a - f32(f32(refl[b]) - f32(1e-9)))
        a = f32(a - f32(f32(refr[b]) - f32(1e-9)))  # presets always carry refr
        survival = f32(f32(1.0) - a)
        always = float(f32(refl[b])) < 1e-4 and float(f32(refr[b])) < 1e-4
        p = None if always else float(f32(refl[b]) / f32(f32(refl[b]) + f32(refr[b])))
        out.append({"survival": float(survival), "always_reflect": always, "p_reflect": p})
    return out


def presets(reference: str):
    path = os.path.join(reference, "blender", "render_EAR", "materials.py")
    spec = importlib.util.spec_from_file_location("ear_reference_materials", path)
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    names = mod.materials()
    res = []
    for key, name, _ in names[1:]:
        refl, refr, spec3 = mod.lookup(key)
        res.append({"name": name, "refl": refl, "refr": refr, "spec": spec3,
                    "derived": derive(refl, refr)})
    return res


def presets_room(pre):
    from ear_gb300 import earfile, scenes

    v = scenes.box_triangles(5.0, 4.0, 3.0)
    mats = [(p["name"], p["refl"], p["refr"], p["spec"]) for p in pre[1:7]]
    meshes = [(mats[i][0], v[2 * i:2 * i + 2]) for i in range(6)]
    return earfile.encode(
        materials=mats, meshes=meshes,
        sources=[{"file": "dry.wav", "location": [1.2, 1.5, 1.4], "gain": 1.0}],
        recorders=[{"file": "mono.wav", "location": [3.9, 2.6, 1.6]},
                   {"file": "stereo.wav", "location": [3.0, 1.0, 1.7], "channels": 2,
                    "right_ear": [0.0, -1.0, 0.0], "head_size": 0.18,
                    "head_absorption": [0.1, 0.3, 0.9]}],
        settings={"debug": 0, "absorption": [0.01, 0.02, 0.05], "drylevel": 1.0,
                  "samples": 10000, "maxthreads": 4})


def oracle_shoebox():
    import oracle
    from ear_gb300 import scenes

    w = scenes.shoebox()
    kw = dict(w.render)
    kw["num_rays"] = 300
    r = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders, threads=1,
                      debug_band=1, debug_rays=300, debug_max_record=50, **kw)
    hit, bt, vis = r["debug"]
    e = (r["hist64"] ** 2).sum(-1)
    return {"config": {"workload": w.name, "rays_per_band": 300, "seed": kw["seed"]},
            "counters": r["counters"],
            "energy": e.tolist(),
            "first_sample": r["first_sample"].tolist(), "last_sample": r["last_sample"].tolist(),
            "hits_sha256": hashlib.sha256(hit.tobytes()).hexdigest(),
            "visible_sha256": hashlib.sha256(vis.tobytes()).hexdigest()}


def main():
    ap = argparse.ArgumentParser()
    default = os.environ.get("EAR_REFERENCE_ROOT") or os.path.join(HERE, "..", "..", "..", "reference")
    ap.add_argument("--reference", default=os.path.normpath(default))
    args = ap.parse_args()
    pre = presets(args.reference)
    with open(os.path.join(HERE, "material_presets.json"), "w") as f:
        json.dump(pre, f, indent=1)
    with open(os.path.join(HERE, "presets_room.ear"), "wb") as f:
        f.write(presets_room(pre))
    with open(os.path.join(HERE, "oracle_shoebox.json"), "w") as f:
        json.dump(oracle_shoebox(), f, indent=1)
    print("wrote fixtures to", HERE)


if __name__ == "__main__":
    main()

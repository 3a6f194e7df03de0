"""Build recipe of the reference-built checkers in oracle/_ref/:

* libear_ref.so -- the reference's own equalizer and WAV sources
  (lib/equalizer/Equalizer.cpp, lib/wave/WaveFile.cpp) behind the C entry
  points of oracle/ref_shim.cpp;
* libear_ref_render.so -- the reference's ray-tracing sources (src/Scene,
  Mesh, Triangle, Material, MonoRecorder, StereoRecorder, Recorder,
  Datatype, Settings, SoundFile, Animated, HelperFunctions) with the same
  two libraries, behind oracle/ref_render.cpp.  GMTL 0.6.1 and Boost.Thread
  are not installed; oracle/refshim/ provides the small part of their
  interface those sources call (written for this project, with the
  oracle's arithmetic and a replayed random tape), and
  oracle/refshim/prelude.h routes pow / powf to the shared portable power
  function.  The sources are compiled where they lie, read through one
  mechanical rewrite: `pointer > 0` tests (ill-formed since C++11 and
  rejected by GCC 13) become `pointer != 0`.  Nothing else changes.  It
  links the oracle library (oracle/_build) for that power function.

TEST INFRASTRUCTURE ONLY.  The outputs are git-ignored; they exist only
where the reference tree does (the GPU machine has none, and the tests that
need them skip there).

    python oracle/build_ref.py [REFERENCE_ROOT]

REFERENCE_ROOT defaults to $EAR_REFERENCE_ROOT, else to a checkout named
``reference`` beside this repository.
"""
from __future__ import annotations

import os
import re
import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref" / "libear_ref.so"
OUT_RENDER = HERE / "_ref" / "libear_ref_render.so"
ORACLE_LIB = HERE / "_build" / "libear_oracle.so"
REF_SOURCES = ["Scene", "Mesh", "Triangle", "Material", "MonoRecorder", "StereoRecorder",
               "Recorder", "Datatype", "Settings", "SoundFile", "Animated", "HelperFunctions"]
# `animation > 0` and the like: ordered comparisons of a pointer with 0
POINTER_GT_ZERO = re.compile(r"\b(mat|animation|mesh|right_ear_animation) > 0\b")


def default_root() -> Path:
    """$EAR_REFERENCE_ROOT, else the ``reference`` checkout beside this
    repository."""
    env = os.environ.get("EAR_REFERENCE_ROOT")
    return Path(env) if env else HERE.parent.parent / "reference"


def build(root: Path | None = None, force: bool = False) -> Path | None:
    root = default_root() if root is None else Path(root)
    eq = root / "lib" / "equalizer" / "Equalizer.cpp"
    wav = root / "lib" / "wave" / "WaveFile.cpp"
    if not (eq.exists() and wav.exists()):
        return None
    srcs = [HERE / "ref_shim.cpp", eq, wav]
    if not force and OUT.exists() and all(OUT.stat().st_mtime >= s.stat().st_mtime for s in srcs):
        return OUT
    OUT.parent.mkdir(parents=True, exist_ok=True)
    tmp = OUT.with_suffix(".so.tmp")
    cxx = shutil.which("g++") or "g++"
    # -ffp-contract=off: the reference's x86 builds round every product.
    # WaveFile.cpp calls fabs without including <math.h> (its Windows build
    # gets it through <windows.h>), so the header is force-included.
    cmd = [cxx, "-O2", "-fPIC", "-shared", "-ffp-contract=off", "-w", "-include", "math.h",
           "-I", str(eq.parent), "-I", str(wav.parent), *map(str, srcs), "-o", str(tmp)]
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed:\n" + r.stdout)
    tmp.replace(OUT)
    return OUT


def _compile_stdin(cxx, text, flags, obj):
    r = subprocess.run([cxx, *flags, "-x", "c++", "-", "-c", "-o", str(obj)], input=text,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference build failed (%s):\n%s" % (obj.name, r.stdout))


def build_render(root: Path | None = None, force: bool = False) -> Path | None:
    """libear_ref_render.so (see the module docstring); None where the
    reference tree or the oracle library is absent."""
    root = default_root() if root is None else Path(root)
    src = root / "src"
    eq = root / "lib" / "equalizer" / "Equalizer.cpp"
    wav = root / "lib" / "wave" / "WaveFile.cpp"
    refs = [src / (n + ".cpp") for n in REF_SOURCES]
    if not all(p.exists() for p in refs + [eq, wav]) or not ORACLE_LIB.exists():
        return None
    shim = HERE / "refshim"
    mine = [HERE / "ref_render.cpp", *sorted(shim.rglob("*.h*"))]
    deps = refs + [eq, wav, ORACLE_LIB] + mine + [Path(__file__)]
    if not force and OUT_RENDER.exists() and all(
            OUT_RENDER.stat().st_mtime >= p.stat().st_mtime for p in deps):
        return OUT_RENDER
    obj_dir = HERE / "_ref" / "obj"
    obj_dir.mkdir(parents=True, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    # C++98 as the reference was written; -ffp-contract=off rounds every
    # product as the oracle does
    flags = ["-std=gnu++98", "-O2", "-fPIC", "-ffp-contract=off", "-w",
             "-include", str(shim / "prelude.h"), "-I", str(shim), "-I", str(src)]
    objs = []
    for p in refs:
        obj = obj_dir / (p.stem + ".o")
        _compile_stdin(cxx, POINTER_GT_ZERO.sub(r"\1 != 0", p.read_text()), flags, obj)
        objs.append(obj)
    for p in (eq, wav):
        obj = obj_dir / (p.stem + ".o")
        r = subprocess.run([cxx, "-O2", "-fPIC", "-ffp-contract=off", "-w", "-include", "math.h",
                            "-I", str(p.parent), "-c", str(p), "-o", str(obj)],
                           stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        if r.returncode != 0:
            raise RuntimeError("reference build failed:\n" + r.stdout)
        objs.append(obj)
    drv = obj_dir / "ref_render.o"
    _compile_stdin(cxx, (HERE / "ref_render.cpp").read_text(), flags, drv)
    tmp = OUT_RENDER.with_suffix(".so.tmp")
    r = subprocess.run([cxx, "-shared", "-o", str(tmp), str(drv), *map(str, objs),
                        "-L", str(ORACLE_LIB.parent), "-lear_oracle",
                        "-Wl,-rpath,$ORIGIN/../_build", "-pthread"],
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference link failed:\n" + r.stdout)
    tmp.replace(OUT_RENDER)
    return OUT_RENDER


if __name__ == "__main__":
    arg = Path(sys.argv[1]) if len(sys.argv) > 1 else None
    print(build(arg))
    print(build_render(arg))

"""Build recipe of oracle/_ref/libear_ref.so: the reference's own
equalizer and WAV sources (lib/equalizer/Equalizer.cpp,
lib/wave/WaveFile.cpp), compiled where they lie in the reference tree,
behind the C entry points of oracle/ref_shim.cpp.

TEST INFRASTRUCTURE ONLY.  The output is git-ignored; it exists only where
the reference tree does (the GPU machine has none, and the tests that need it
skip there).  The rest of the reference (src/) needs GMTL and Boost, which
are not present, so it is not built.

    python oracle/build_ref.py [REFERENCE_ROOT]
"""
from __future__ import annotations

import shutil
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref" / "libear_ref.so"
DEFAULT_ROOT = Path("/root/reference")


def build(root: Path = DEFAULT_ROOT, force: bool = False) -> Path | None:
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


if __name__ == "__main__":
    print(build(Path(sys.argv[1]) if len(sys.argv) > 1 else DEFAULT_ROOT))

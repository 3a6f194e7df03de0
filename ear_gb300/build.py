"""Build the sm_103a extension library, the CPU restatement (oracle) and the
``EAR`` command-line host, in-tree and in parallel.

    python -m ear_gb300.build            # build what is out of date
    python -m ear_gb300.build --force    # rebuild everything

Outputs (all git-ignored): ``ear_gb300/lib/libear_gb300.so``,
``ear_gb300/bin/EAR`` and ``oracle/_build/libear_oracle.so``.  A stamp
file holds a hash of the sources, flags and machine so repeated calls are
no-ops.  nvcc cross-compiles for sm_103a without a GPU.
"""
from __future__ import annotations

import hashlib
import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent
PKG = ROOT / "ear_gb300"
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "lib" / "libear_gb300.so"
CLI = PKG / "bin" / "EAR"
ORACLE_SRC = ROOT / "oracle" / "ear_oracle.cpp"
ORACLE_LIB = ROOT / "oracle" / "_build" / "libear_oracle.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -ffp-contract=off: host code must round like the CPU restatement (on
# aarch64 gcc would otherwise fuse a*b+c into fmadd).
HOSTFLAGS = ["-Xcompiler", "-fPIC,-ffp-contract=off,-O2"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr"] + ARCH + HOSTFLAGS

# (source, extra nvcc flags).  --fmad=false wherever results must be
# bit-identical to the CPU restatement.
CUDA_UNITS = [
    ("bvh_build.cu", ["--fmad=false"]),
    ("trace_exact.cu", ["--fmad=false"]),
    ("trace_fast.cu", ["--fmad=true", "-prec-div=false"]),
    ("api.cu", ["--fmad=false"]),
    ("batch.cu", ["--fmad=false"]),
    ("vismap.cu", ["--fmad=false"]),
    # exact paths use explicit _rn intrinsics; the FFT may contract
    ("aural.cu", ["--fmad=true"]),
]
CLI_SOURCES = ["cli/ear_cli.cpp", "cli/earfile.cpp", "cli/wavefile.cpp"]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _hash(paths, extra: str) -> str:
    h = hashlib.sha256(extra.encode())
    for p in sorted(paths):
        h.update(str(p).encode())
        h.update(Path(p).read_bytes())
    return h.hexdigest()


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n%s\n%s" % (" ".join(map(str, cmd)), r.stdout))
    return r.stdout


def _stamp_ok(stamp: Path, digest: str, outputs) -> bool:
    return stamp.exists() and stamp.read_text() == digest and all(Path(o).exists() for o in outputs)


def build_library(force: bool = False, verbose: bool = False) -> Path:
    srcs = [CSRC / u for u, _ in CUDA_UNITS] + sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h"))
    srcs.append(ROOT / "include" / "ear_gb300.h")
    digest = _hash(srcs, " ".join(NVFLAGS) + platform.machine() + str(CUDA_UNITS))
    stamp = BUILD / "lib.stamp"
    if not force and _stamp_ok(stamp, digest, [LIB]):
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    LIB.parent.mkdir(parents=True, exist_ok=True)
    nv = nvcc()

    def compile_unit(unit):
        src, extra = unit
        obj = BUILD / (Path(src).stem + ".o")
        cmd = [nv, *NVFLAGS, *extra, "-I", str(ROOT / "include"), "-c", str(CSRC / src), "-o", str(obj)]
        if verbose:
            cmd += ["-Xptxas", "-v"]
        out = _run(cmd)
        if verbose and out:
            print(out)
        return obj

    with ThreadPoolExecutor(max_workers=len(CUDA_UNITS)) as ex:
        objs = list(ex.map(compile_unit, CUDA_UNITS))
    tmp = LIB.with_suffix(".so.tmp")
    _run([nv, "-shared", *ARCH, "-o", str(tmp), *map(str, objs)])
    os.replace(tmp, LIB)
    stamp.write_text(digest)
    return LIB


def build_oracle(force: bool = False) -> Path:
    digest = _hash([ORACLE_SRC, ROOT / "include" / "ear_gb300.h"], platform.machine())
    stamp = ORACLE_LIB.parent / "oracle.stamp"
    if not force and _stamp_ok(stamp, digest, [ORACLE_LIB]):
        return ORACLE_LIB
    ORACLE_LIB.parent.mkdir(parents=True, exist_ok=True)
    tmp = ORACLE_LIB.with_suffix(".so.tmp")
    cxx = shutil.which("g++") or "g++"
    _run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
          "-pthread", str(ORACLE_SRC), "-o", str(tmp)])
    os.replace(tmp, ORACLE_LIB)
    stamp.write_text(digest)
    return ORACLE_LIB


def build_cli(force: bool = False) -> Path | None:
    srcs = [CSRC / s for s in CLI_SOURCES]
    if not all(s.exists() for s in srcs):
        return None
    hdrs = sorted((CSRC / "cli").glob("*.h"))
    digest = _hash(srcs + hdrs + [ROOT / "include" / "ear_gb300.h"], platform.machine())
    stamp = BUILD / "cli.stamp"
    if not force and _stamp_ok(stamp, digest, [CLI]):
        return CLI
    BUILD.mkdir(parents=True, exist_ok=True)
    CLI.parent.mkdir(parents=True, exist_ok=True)
    cxx = shutil.which("g++") or "g++"
    tmp = CLI.with_suffix(".tmp")
    _run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", str(ROOT / "include"),
          *map(str, srcs), "-o", str(tmp), "-L", str(LIB.parent), "-lear_gb300",
          "-Wl,-rpath,$ORIGIN/../lib", "-pthread"])
    os.replace(tmp, CLI)
    stamp.write_text(digest)
    return CLI


def build_all(force: bool = False, verbose: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f_lib = ex.submit(build_library, force, verbose)
        f_or = ex.submit(build_oracle, force)
        f_lib.result()
        f_or.result()
    build_cli(force)


if __name__ == "__main__":
    build_all(force="--force" in sys.argv, verbose="-v" in sys.argv)
    print("built", LIB, ORACLE_LIB, CLI if CLI.exists() else "(no CLI)")

"""The C-ABI library loads without a GPU, exports every function declared
in include/ear_gb300.h, its ctypes mirror matches the C layout, and the
host-only functions agree with the oracle's restatement."""
import ctypes as C
import re
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

import oracle
from ear_gb300 import _native as N

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = set()
    for h in HEADERS:
        text = h.read_text()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^[a-z_0-9 \*]*?\b(ear_[a-z_0-9]+)\s*\(", text, flags=re.M):
            names.add(m.group(1))
    return sorted(names)


def test_library_exports_every_declared_symbol():
    L = N.lib()
    names = declared_functions()
    assert "ear_render" in names and "ear_scene_create" in names
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    assert set(names) <= set(N.SIGNATURES), set(names) - set(N.SIGNATURES)


def test_ctypes_layout_matches_c():
    """Compile a probe with the system C compiler and compare sizeof/offsetof."""
    structs = {
        "ear_material": N.EarMaterial, "ear_scene_desc": N.EarSceneDesc,
        "ear_bvh_opts": N.EarBvhOpts, "ear_recorder": N.EarRecorder, "ear_source": N.EarSource,
        "ear_render_params": N.EarRenderParams, "ear_render_stats": N.EarRenderStats,
        "ear_histograms": N.EarHistograms, "ear_batch_job": N.EarBatchJob,
        "ear_batch_config": N.EarBatchConfig, "ear_tune_opts": N.EarTuneOpts,
        "ear_tune_result": N.EarTuneResult, "ear_conv_context": N.EarConvContext,
        "ear_conv_stats": N.EarConvStats,
    }
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "ear_gb300.h"', "int main(){"]
    for cname, py in structs.items():
        lines.append(f'printf("{cname} %zu\\n", sizeof({cname}));')
        for fname, _ in py._fields_:
            lines.append(f'printf("{cname}.{fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("return 0;}")
    with tempfile.TemporaryDirectory() as d:
        src = Path(d) / "probe.c"
        src.write_text("\n".join(lines))
        exe = Path(d) / "probe"
        subprocess.run(["gcc", "-I", str(ROOT / "include"), str(src), "-o", str(exe)], check=True)
        out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    got = dict(line.rsplit(" ", 1) for line in out.strip().splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == C.sizeof(py), cname
        for fname, _ in py._fields_:
            assert int(got[f"{cname}.{fname}"]) == getattr(py, fname).offset, (cname, fname)


def test_version_and_errors_without_gpu():
    L = N.lib()
    assert L.ear_abi_version() == 2
    assert b"sm_103a" in L.ear_version()
    h = C.c_void_p()
    assert L.ear_scene_create(None, C.byref(h)) == N.EAR_ERR_INVALID_ARG
    assert L.ear_last_error()


def test_invalid_material_is_rejected_before_device_work():
    from ear_gb300 import Material

    v = np.zeros((1, 9), np.float32)
    mats = (N.EarMaterial * 1)(Material(reflection=(0.9, 0.9, 0.9), refraction=(0.5, 0.5, 0.5)).to_c())
    ids = np.zeros(1, np.int32)
    d = N.EarSceneDesc(1, v.ctypes.data_as(C.POINTER(C.c_float)),
                       ids.ctypes.data_as(C.POINTER(C.c_int32)), 1, mats, 0)
    h = C.c_void_p()
    assert N.lib().ear_scene_create(C.byref(d), C.byref(h)) == N.EAR_ERR_INVALID_ARG
    assert b"Invalid material" in N.lib().ear_last_error()


def test_track_functions_match_oracle():
    """ear_track_* (library host code) == the oracle's FloatBuffer restatement."""
    rng = np.random.default_rng(1)
    x = (rng.standard_normal(5000) * np.exp(-np.arange(5000) / 800.0)).astype(np.float32)
    x[:100] = 0
    x[100] = 3.0
    first, last = 100, 4900
    a, b = x.copy(), x.copy()
    N.check(N.lib().ear_track_power(a.ctypes.data, first, last, 0.335))
    oracle.lib().oracle_track_power(b.ctypes.data, first, last, 0.335)
    np.testing.assert_array_equal(a, b)
    assert N.lib().ear_track_maximum(a.ctypes.data, first, last) == \
        oracle.lib().oracle_track_maximum(b.ctypes.data, first, last)
    for tr in (-1.0, 0.01, 0.5):
        assert N.lib().ear_track_length(a.ctypes.data, len(a), first, last, tr) == \
            oracle.lib().oracle_track_length(b.ctypes.data, len(b), first, last, tr)
    assert N.lib().ear_track_t60(a.ctypes.data, first, last) == \
        oracle.lib().oracle_track_t60(b.ctypes.data, first, last)


def test_sah_cost_arguments_are_checked_before_device_work():
    c = C.c_double()
    assert N.lib().ear_scene_sah_cost(None, 4, 1.0, 1.0, C.byref(c)) == N.EAR_ERR_INVALID_ARG


def test_batch_arguments_are_checked_before_device_work():
    h = C.c_void_p()
    p = N.EarRenderParams()
    assert N.lib().ear_batch_create(None, 0, None, 0, C.byref(p), C.byref(h)) == N.EAR_ERR_INVALID_ARG
    assert N.lib().ear_batch_run(None, None) == N.EAR_ERR_INVALID_ARG
    assert N.lib().ear_batch_tune(None, None, None) == N.EAR_ERR_INVALID_ARG


def test_header_is_plain_c():
    """include/ear_gb300.h compiles as C99 and as C++11 on its own: the
    boundary holds no C++ or CUDA types, so a C, cgo or ctypes binding can
    include it."""
    import shutil
    import subprocess

    root = Path(__file__).resolve().parent.parent
    hdr = str(root / "include" / "ear_gb300.h")
    for cc, std, lang in (("gcc", "-std=c99", "c"), ("g++", "-std=c++11", "c++")):
        exe = shutil.which(cc)
        if exe is None:
            pytest.skip(cc + " not found")
        r = subprocess.run([exe, std, "-Wall", "-Wextra", "-Werror", "-fsyntax-only", "-x", lang, hdr],
                           capture_output=True, text=True, timeout=120)
        assert r.returncode == 0, r.stderr


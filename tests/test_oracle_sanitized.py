"""The CPU restatement under AddressSanitizer and UndefinedBehaviorSanitizer:
tests/oracle_sanitize_main.cpp includes the oracle's source and drives
render, debug record, adjoint, area emitter, empty and one-triangle scenes
and the random tape; any out-of-bounds access, leak, overflow or other
undefined behaviour ends the run with a report and a non-zero status."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def test_oracle_is_clean_under_asan_and_ubsan(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = tmp_path / "oracle_sanitized"
    cmd = [cxx, "-std=c++17", "-O1", "-g", "-fsanitize=address,undefined",
           "-fno-sanitize-recover=all", "-ffp-contract=off", "-I", str(ROOT / "include"),
           str(ROOT / "tests" / "oracle_sanitize_main.cpp"), "-o", str(exe), "-pthread"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    if r.returncode != 0 and "sanitize" in (r.stderr or "") and "cannot find" in (r.stderr or ""):
        pytest.skip("the sanitizer runtimes are not installed")
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=600)
    assert run.returncode == 0, run.stdout + run.stderr
    assert "runtime error" not in run.stderr and "ERROR: AddressSanitizer" not in run.stderr
    assert run.stdout.startswith("ok energy")

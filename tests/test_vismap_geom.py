"""Conservativeness of the listener visibility maps, checked on the CPU.

tests/vismap_geom_check.cu compiles the maps' own geometry
(ear_gb300/csrc/vismap_geom.h: the cells of a padded box, of a projected
triangle and of a query direction, and the walk's distance cut) for the
host and samples points where the triangle test could report a hit; every
such point's visibility test must read a cell that lists the triangle, and
must not stop before its entry.  The GPU tests check the same end to end,
bit-exact against the oracle.  (With the projected triangle's widening
removed, the same check reports misses.)
"""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def _nvcc():
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    return None


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    out = tmp_path_factory.mktemp("vismap") / "vismap_geom_check"
    cmd = [nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I", str(ROOT / "include"),
           "-x", "cu", str(ROOT / "tests" / "vismap_geom_check.cu"), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_every_hit_point_reads_a_cell_listing_its_triangle(checker, seed):
    r = subprocess.run([str(checker), "200000", str(seed)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    line = r.stdout.strip().splitlines()[-1]
    fields = dict(zip(line.split()[0::2], line.split()[1::2]))
    assert int(fields["queries"]) > 1_500_000
    assert int(fields["projected"]) > 1_000_000  # the projected-triangle test is exercised
    assert int(fields["misses"]) == 0 and int(fields["cut_misses"]) == 0

"""Conservativeness of the listener visibility maps, checked on the CPU.

tests/vismap_geom_check.cu compiles the maps' own geometry
(ear_gb300/csrc/vismap_geom.h: the cells of a padded box, of a projected
triangle and of a query direction, and the walk's distance cut) for the
host and samples points where the triangle test could report a hit; every
such point's visibility test must read a cell that lists the triangle, and
must not stop before its entry.  (With the projected triangle's widening
removed, that check reports misses.)

tests/vismap_walk_check.cu then compares, on seeded random scenes of ~150
triangles, the visibility test answered from the cell lists with the
brute-force any-hit test over all triangles, for vertices on triangles,
in free space and beyond triangle edges and corners, with both evaluation
orders of the triangle test.  (With the walk's distance cut shortened by
2%, that check reports mismatches.)  The GPU tests check the same end to
end, bit-exact against the oracle.
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


def _build(tmp_path_factory, name):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    out = tmp_path_factory.mktemp("vismap") / name
    cmd = [nvcc, "-std=c++17", "-O2", "-Xcompiler", "-ffp-contract=off",
           "-gencode", "arch=compute_103a,code=sm_103a", "-I", str(ROOT / "include"),
           "-x", "cu", str(ROOT / "tests" / (name + ".cu")), "-o", str(out)]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return out


def _fields(stdout):
    line = stdout.strip().splitlines()[-1]
    return dict(zip(line.split()[0::2], line.split()[1::2]))


@pytest.fixture(scope="module")
def checker(tmp_path_factory):
    return _build(tmp_path_factory, "vismap_geom_check")


@pytest.fixture(scope="module")
def walker(tmp_path_factory):
    return _build(tmp_path_factory, "vismap_walk_check")


@pytest.mark.parametrize("seed", [1, 2, 3])
def test_every_hit_point_reads_a_cell_listing_its_triangle(checker, seed):
    r = subprocess.run([str(checker), "200000", str(seed)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = _fields(r.stdout)
    assert int(fields["queries"]) > 1_500_000
    assert int(fields["projected"]) > 1_000_000  # the projected-triangle test is exercised
    assert int(fields["misses"]) == 0 and int(fields["cut_misses"]) == 0


@pytest.mark.parametrize("seed", [1, 2])
def test_map_walk_equals_the_brute_force_visibility_test(walker, seed):
    r = subprocess.run([str(walker), "3000", str(seed)], capture_output=True, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    fields = _fields(r.stdout)
    queries, blocked = int(fields["queries"]), int(fields["blocked"])
    assert queries > 100_000 and 0.2 * queries < blocked < 0.8 * queries
    assert int(fields["mismatches"]) == 0
    print("reported hits: point at t", fields["worst_outside_over_pad"],
          "x box_pad outside the box, exact crossing", fields["worst_crossing_over_pad"],
          "x box_pad, crossing parameter", fields["worst_t_beyond"], "beyond [0, 1]")
    # the lists test a small part of the triangles the brute force tests
    assert int(fields["map_tests"]) * 10 < int(fields["brute_tests"])

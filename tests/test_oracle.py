"""CPU tests of the restatement oracle: published known-answer vectors,
analytic checks and internal consistency.  The reference ships no tests or
golden vectors for this path, so these are the pins (parity against the
reference binary itself is unpinned; see oracle/ear_oracle.cpp)."""
import math
import os

import numpy as np
import pytest

import oracle
from ear_gb300 import Material, Recorder, Source, scenes

THREADS = max(1, min(8, os.cpu_count() or 1))


# Philox-4x32-10 known-answer vectors published with Random123 (Salmon et
# al., SC'11): (counter, key) -> output.
PHILOX_KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]),
    ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2, [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]),
    ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0],
     [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]),
]


@pytest.mark.parametrize("ctr,key,expect", PHILOX_KAT)
def test_philox_kat(ctr, key, expect):
    assert oracle.philox(ctr, key) == expect


def test_portable_pow_accuracy():
    """portable_powf stays within a few ulp of libm on the path's domain:
    bases in (0, 1] (air factors, lobe cosines, head absorption) and
    exponents up to 1000."""
    rng = np.random.default_rng(0)
    xs = np.concatenate([rng.uniform(0.0, 1.0, 4000), 1 - rng.uniform(0, 0.05, 4000),
                         rng.uniform(0.5, 2.0, 2000)]).astype(np.float32)
    ys = np.concatenate([rng.uniform(0, 1000, 4000), rng.uniform(0, 400, 4000),
                         rng.uniform(0, 8, 2000)]).astype(np.float32)
    worst = 0.0
    for x, y in zip(xs, ys):
        got = oracle.powf(float(x), float(y))
        ref = math.pow(float(x), float(y))
        if ref < 1e-30 or ref > 1e30:
            continue
        err = abs(got - ref) / ref
        # relative error budget: a few float ulps times |y log2 x| + 2
        budget = 2.4e-7 * (abs(float(y) * math.log2(float(x))) + 4.0)
        assert err <= budget, (x, y, got, ref)
        worst = max(worst, err)
    assert oracle.powf(1.0, 1234.5) == 1.0
    assert oracle.powf(0.0, 3.0) == 0.0
    assert oracle.powf(0.7, 0.0) == 1.0


def test_material_derivation_matches_reference_formula():
    """Material::Material stores survival = refl + refr - 2e-9 through
    1 - (1 - (f - 1e-9f) - (r - 1e-9f)) in float (src/Material.cpp:33-60);
    Material::Bounce reflects with probability refl / (refl + refr)."""
    import ctypes as C

    def f32(x):
        return float(np.float32(x))

    for refl, refr in [((0.9, 0.8, 0.7), None), ((0.6, 0.7, 0.8), (0.39, 0.24, 0.17)),
                       ((0.0, 0.0, 0.00005), (0.00005, 0.5, 0.0))]:
        m = Material(reflection=refl, refraction=refr, specularity=(0.1, 0.2, 0.3))
        surv = (C.c_float * 3)()
        prob = (C.c_float * 3)()
        alw = (C.c_int32 * 3)()
        spec = (C.c_float * 3)()
        rc = oracle.lib().oracle_material(C.byref(m.to_c()), surv, prob, alw, spec)
        assert rc == 0
        for b in range(3):
            a = np.float32(1.0)
            a = np.float32(a - np.float32(np.float32(refl[b]) - np.float32(1e-9)))
            fr = refr[b] if refr else 0.0
            if refr:
                a = np.float32(a - np.float32(np.float32(fr) - np.float32(1e-9)))
            assert surv[b] == f32(np.float32(1.0) - a)
            assert bool(alw[b]) == (f32(refl[b]) < 1e-4 and f32(fr) < 1e-4)
            if not alw[b]:
                assert prob[b] == f32(np.float32(refl[b]) / np.float32(np.float32(refl[b]) + np.float32(fr)))


def test_closest_hit_tie_takes_lowest_index():
    """Mesh::RayIntersection keeps the first of equal-t hits (strict <,
    src/Mesh.cpp:40)."""
    t = np.array([[0, 0, 0, 1, 0, 0, 0, 1, 0]], np.float32)
    v = np.concatenate([t, t, t], 0) + np.array([0, 0, 1, 0, 0, 1, 0, 0, 1], np.float32)
    v[0, [2, 5, 8]] = 2.0  # farther copy first
    o = np.array([[0.2, 0.2, 0.0]], np.float32)
    d = np.array([[0.0, 0.0, 1.0]], np.float32)
    hit, tt = oracle.closest_hit(v, o, d)
    assert hit[0] == 1 and tt[0] == 1.0
    # a hit closer than 0.001 is ignored
    hit, _ = oracle.closest_hit(v, np.array([[0.2, 0.2, 0.9995]], np.float32), d)
    assert hit[0] == 0


def test_segment_interval():
    """Mesh::LineIntersection: blocked only for 1e-5 < t < 1 (src/Mesh.cpp:65)."""
    tri = np.array([[0, 0, 1, 1, 0, 1, 0, 1, 1]], np.float32)
    o = np.array([[0.2, 0.2, 0.0], [0.2, 0.2, 0.0], [0.2, 0.2, 1.0]], np.float32)
    d = np.array([[0, 0, 2.0], [0, 0, 0.999], [0, 0, 1.0]], np.float32)
    assert list(oracle.segment_blocked(tri, o, d)) == [True, False, False]


def test_shoebox_first_order_reflections_arrive_at_image_source_times():
    """Fully specular shoebox: the earliest non-direct contribution comes from
    a first-order image source (arrival time |x - image| / 343)."""
    w = scenes.shoebox(num_rays=20000)
    kw = dict(w.render)
    kw["bands"] = (0,)
    r = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders, threads=4,
                      no_direct=True, **kw)
    h = r["hist64"][0, 0]
    nz = np.flatnonzero(h)
    assert nz.size > 0
    src = np.array([2.0, 3.5, 1.5])
    rec = np.array([7.0, 3.5, 1.5])
    dims = np.array([10.0, 7.0, 4.0])
    images = []
    for ax in range(3):
        for wall in (0.0, dims[ax]):
            im = src.copy()
            im[ax] = 2 * wall - src[ax]
            images.append(np.linalg.norm(rec - im))
    first_bin = int(min(images) / 343.0 * 44100)
    # the triangular splat of a contribution starts at its arrival bin
    assert abs(int(nz[0]) - first_bin) <= 2, (nz[0], first_bin)


def test_threading_does_not_change_paths():
    w = scenes.small_test_room()
    kw = dict(w.render)
    kw["num_rays"] = 600
    a = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders, threads=1, **kw)
    b = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders, threads=5, **kw)
    assert a["counters"] == b["counters"]
    np.testing.assert_array_equal(a["first_sample"], b["first_sample"])
    np.testing.assert_array_equal(a["last_sample"], b["last_sample"])
    np.testing.assert_allclose(a["hist64"], b["hist64"], rtol=1e-12, atol=1e-18)


def test_direct_sound_and_scaling():
    """Empty scene: only the direct lobe, INV_SPHERE_2(len) * air^len * dry
    splatted at len / 343 s, then scaled by gain^2 (src/Scene.cpp:299-314)."""
    src = Source(location=np.array([0.0, 0.0, 0.0], np.float32), gain=2.0)
    rec = Recorder(location=np.array([3.0, 4.0, 0.0], np.float32))
    r = oracle.render(np.zeros((0, 9), np.float32), np.zeros(0, np.int32),
                      [Material(reflection=(0.5, 0.5, 0.5))], src, [rec], num_rays=10,
                      num_bins=44100, air_absorption=(0.0, 0.0, 0.0), dry=0.5, max_bounces=5)
    h = r["hist64"][0, 0]
    s = int(np.float32(5.0) / np.float32(343.0) * 44100.0)
    w = math.ceil(math.sqrt(5.0))
    a = 1.0 / (4 * 3.14159265 * 25.0) * 0.5
    ampl = 2 * a / math.sqrt(5.0)
    assert np.flatnonzero(h).tolist() == list(range(s, s + w))
    # first bins scaled by gain^2 = 4; the last written bin is skipped by
    # FloatBuffer::Multiply's [first_sample, real_length) range
    assert h[s] == pytest.approx(4 * ampl, rel=1e-6)
    assert h[s + w - 1] == pytest.approx(ampl / w, rel=1e-5)
    assert r["first_sample"][0, 0] == s and r["last_sample"][0, 0] == s + w - 1


def test_sabine_eyring_shoebox():
    """src/EAR.cpp:271-284 on the 10x7x4 shoebox: V = 280, S = 276."""
    import ctypes as C

    from ear_gb300 import _native as N

    w = scenes.shoebox()
    out = np.zeros(5, np.float32)
    blocks = np.array([12], np.int64)
    m = w.materials[0].to_c()
    N.check(N.lib().ear_statistical_t60(w.vertices.ctypes.data, blocks.ctypes.data, 1,
                                        C.byref(m), 0.0, out.ctypes.data))
    V, S, A, sab, eyr = out
    assert V == pytest.approx(280.0, rel=1e-5)
    assert S == pytest.approx(276.0, rel=1e-5)
    assert A == pytest.approx(276.0 * 0.2, rel=1e-4)
    assert sab == pytest.approx(0.1611 * 280 / (276 * 0.2), rel=1e-4)
    assert eyr == pytest.approx(0.1611 * 280 / (-276 * math.log(0.8)), rel=1e-4)


def _opaque(a, spec=0.5):
    return [Material(reflection=tuple((1.0 - a[i]).tolist()), specularity=(spec,) * 3, name=f"m{i}")
            for i in range(len(a))]


def test_oracle_adjoint_pathwise_matches_central_differences():
    """The FP64 path-replay gradient of sum(g * h) for opaque materials (no
    parameter-dependent random choice) equals central differences with the
    same random numbers, after the 1/N and gain^2 finalize scaling."""
    w, _, _ = scenes.inverse_shoebox()
    a = np.full((8, 3), 0.2)
    kw = dict(w.render, num_rays=1500, num_bins=20000)
    g = np.random.default_rng(3).standard_normal((1, 3, kw["num_bins"]))
    grad = oracle.adjoint(w.vertices, w.material_ids, _opaque(a), w.source, w.recorders, g,
                          threads=THREADS, **kw)

    def loss(aa):
        h = oracle.render(w.vertices, w.material_ids, _opaque(aa), w.source, w.recorders,
                          threads=THREADS, **kw)["hist64"]
        return float((h * g).sum())

    for m, b in [(0, 0), (5, 2)]:
        ap, am = a.copy(), a.copy()
        ap[m, b] += 1e-3
        am[m, b] -= 1e-3
        fd = (loss(ap) - loss(am)) / 2e-3
        assert grad[m, b, 0] == pytest.approx(fd, rel=1e-3)


def test_oracle_adjoint_raw_and_scaled_differ_by_the_finalize_scaling():
    """With g nonzero only on bins that the direct sound leaves alone, the
    gradient of the finalized histogram is gain^2 / N times the raw one."""
    w, _, _ = scenes.inverse_shoebox()
    mats = [Material(reflection=(0.7, 0.7, 0.7), refraction=(0.1, 0.1, 0.1),
                     specularity=(0.5,) * 3, name=f"m{i}") for i in range(8)]
    kw = dict(w.render, num_rays=500, num_bins=20000)
    g = np.zeros((1, 3, kw["num_bins"]))
    g[..., 3000:15000] = np.random.default_rng(4).standard_normal((1, 3, 12000))
    raw = oracle.adjoint(w.vertices, w.material_ids, mats, w.source, w.recorders, g,
                         threads=THREADS, raw=True, **kw)
    fin = oracle.adjoint(w.vertices, w.material_ids, mats, w.source, w.recorders, g,
                         threads=THREADS, **kw)
    assert np.abs(raw).max() > 0
    np.testing.assert_allclose(fin, raw / kw["num_rays"], rtol=1e-6, atol=1e-12 * np.abs(raw).max())


def test_split_by_ray_range_sums_to_the_unsplit_render():
    """Rays first_ray .. first_ray+N-1 of the same stream: two halves with
    raw histograms add up to the whole (FP64 re-accumulation)."""
    w = scenes.small_test_room()
    kw = dict(w.render, num_rays=600, raw=True)
    whole = oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders,
                          threads=THREADS, **kw)
    parts = [oracle.render(w.vertices, w.material_ids, w.materials, w.source, w.recorders,
                           threads=THREADS, **dict(kw, num_rays=300, first_ray=f))
             for f in (0, 300)]
    np.testing.assert_allclose(parts[0]["hist64"] + parts[1]["hist64"], whole["hist64"],
                               rtol=1e-12, atol=1e-12 * np.abs(whole["hist64"]).max())
    for k in whole["counters"]:
        assert parts[0]["counters"][k] + parts[1]["counters"][k] == whole["counters"][k]
    assert (np.minimum(parts[0]["first_sample"], parts[1]["first_sample"]) == whole["first_sample"]).all()
    assert (np.maximum(parts[0]["last_sample"], parts[1]["last_sample"]) == whole["last_sample"]).all()

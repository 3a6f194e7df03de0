"""Path-replay adjoint (ear_render_adjoint) and the torch.autograd binding.

1. The kernel's gradient equals the oracle's FP64 gradient of the same
   estimator on the same paths (exact kernels), within float accumulation.
2. For opaque materials the estimator is purely pathwise (no random
   choices depend on the parameters) and equals central finite differences
   with common random numbers to <= 1e-3 relative.
3. The autograd Function routes the EDC loss through the same adjoint.
"""
import os

import numpy as np
import pytest

import oracle
from ear_gb300 import Material, Tracer, scenes

pytestmark = pytest.mark.gpu
THREADS = max(1, min(16, os.cpu_count() or 1))


def _mats(a, r, spec=0.5):
    return [Material(reflection=tuple(1.0 - a[i] - r[i]), refraction=tuple(r[i]),
                     specularity=(spec, spec, spec), name=f"m{i}") for i in range(len(a))]


def _oracle_adjoint(w, mats, g, **kw):
    return oracle.adjoint(w.vertices, w.material_ids, mats, w.source, w.recorders, g,
                          threads=THREADS, **kw)


@pytest.mark.parametrize("raw", [False, True])
def test_adjoint_matches_oracle_fp64(raw):
    w, _, _ = scenes.inverse_shoebox()
    a = np.full((8, 3), 0.2)
    r = np.full((8, 3), 0.05)
    mats = _mats(a, r)
    kw = dict(w.render, num_rays=20000, num_bins=20000, raw=raw, exact=True)
    g = np.random.default_rng(1).standard_normal((1, 3, kw["num_bins"])).astype(np.float32) * 1e3
    with Tracer(w.vertices, w.material_ids, mats) as tr:
        fwd = tr.render(w.source, w.recorders, **kw)
        grad, st = tr.render_adjoint(w.source, w.recorders, g, first=fwd.first_sample,
                                     last=fwd.last_sample, raw_first=fwd.raw_first_sample,
                                     raw_last=fwd.raw_last_sample, **kw)
    assert st["segments"] == fwd.stats["segments"]  # the same paths were re-traced
    ref = _oracle_adjoint(w, mats, g.astype(np.float64), **kw)
    scale = np.abs(ref).max()
    assert scale > 0
    np.testing.assert_allclose(grad, ref, rtol=2e-4, atol=2e-5 * scale)


def test_pathwise_gradient_matches_central_differences():
    """Opaque materials: d/d(absorption) of sum(g * h) by the GPU adjoint
    equals central differences (step 1e-3, common random numbers) to 1e-3.
    The differenced losses are FP64 re-accumulations of the same paths (the
    oracle: exact kernels trace bit-identical paths), because float atomics
    accumulate the GPU histograms in a varying order whose rounding is close
    to the 1e-3-step difference itself."""
    w, _, _ = scenes.inverse_shoebox()
    a = np.full((8, 3), 0.2)
    r = np.zeros((8, 3))
    kw = dict(w.render, num_rays=20000, num_bins=30000, exact=True)
    # positive weights: the loss is not a cancelling sum, so the float
    # atomics' rounding (order-dependent) stays far below the FD numerator
    g = np.random.default_rng(2).uniform(0.5, 1.5, (1, 3, kw["num_bins"])).astype(np.float32) * 1e3
    with Tracer(w.vertices, w.material_ids, _mats(a, r)) as tr:
        fwd = tr.render(w.source, w.recorders, **kw)
        grad, _ = tr.render_adjoint(w.source, w.recorders, g, first=fwd.first_sample,
                                    last=fwd.last_sample, raw_first=fwd.raw_first_sample,
                                    raw_last=fwd.raw_last_sample, **kw)

        def loss(aa):
            h = oracle.render(w.vertices, w.material_ids, _mats(aa, r), w.source, w.recorders,
                              threads=THREADS, **kw)["hist64"]
            return float((h * g.astype(np.float64)).sum())

        h = 1e-3
        for m, b in [(0, 0), (3, 1), (6, 2), (1, 1)]:
            ap, am = a.copy(), a.copy()
            ap[m, b] += h
            am[m, b] -= h
            fd = (loss(ap) - loss(am)) / (2 * h)
            assert abs(grad[m, b, 0] - fd) <= 1e-3 * abs(fd), (m, b, grad[m, b, 0], fd)


def test_autograd_edc_loss():
    torch = pytest.importorskip("torch")
    from ear_gb300 import post
    from ear_gb300.autograd import edc_loss, render_materials

    w, hid_a, hid_r = scenes.inverse_shoebox()
    kw = dict(w.render, num_rays=50000, num_bins=30000)
    spec = np.full((8, 3), 0.5)
    with Tracer(w.vertices, w.material_ids, _mats(hid_a, hid_r)) as tr:
        target = tr.render(w.source, w.recorders, exact=True, **dict(kw, seed=99)).hist
        tgt = torch.stack([post.edc_db_torch(torch.from_numpy(target[0, b]).cuda())
                           for b in range(3)])
        a = torch.full((8, 3), 0.2, dtype=torch.float64, requires_grad=True)
        r = torch.full((8, 3), 0.05, dtype=torch.float64, requires_grad=True)
        hist = render_materials(a, r, tr, w.source, w.recorders, spec, **kw)
        loss = edc_loss(hist, tgt)
        loss.backward()
        assert torch.isfinite(loss) and a.grad is not None and r.grad is not None
        assert a.grad.abs().sum() > 0
        # the same gradient through the raw adjoint call with torch's dL/dh
        hist2 = render_materials(a.detach(), r.detach(), tr, w.source, w.recorders, spec, **kw)
        hist2.requires_grad_(True)
        edc_loss(hist2, tgt).backward()
        fwd = tr.render(w.source, w.recorders, exact=True, **kw)
        g2, _ = tr.render_adjoint(w.source, w.recorders, hist2.grad.float(), first=fwd.first_sample,
                                  last=fwd.last_sample, raw_first=fwd.raw_first_sample,
                                  raw_last=fwd.raw_last_sample, exact=True, **kw)
        np.testing.assert_allclose(a.grad.numpy(), g2[..., 0], rtol=1e-6, atol=1e-12)
        np.testing.assert_allclose(r.grad.numpy(), g2[..., 1], rtol=1e-6, atol=1e-12)

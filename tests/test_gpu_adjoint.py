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


def _seed_fd_setup():
    torch = pytest.importorskip("torch")
    from ear_gb300 import post

    w, hid_a, hid_r = scenes.inverse_shoebox()
    kw = dict(w.render, num_rays=1_000_000, num_bins=60000)
    tr = Tracer(w.vertices, w.material_ids, _mats(hid_a, hid_r))
    target = tr.render(w.source, w.recorders, exact=True, **dict(kw, seed=99)).hist
    tgt = torch.stack([post.edc_db_torch(torch.from_numpy(target[0, b]).cuda()) for b in range(3)])
    return torch, w, kw, tr, tgt


def _assert_seed_mean_agrees(g, f, params, k):
    """Per-seed adjoint gradients g and difference quotients f: the mean
    difference within 3 standard errors (plus 2% of the mean gradient) of
    zero, and the mean gradient standing out of its own noise."""
    for j, p in enumerate(params):
        d = g[:, j] - f[:, j]
        se_d = d.std(ddof=1) / np.sqrt(k)
        mean_g = g[:, j].mean()
        assert abs(mean_g) > 3.0 * g[:, j].std(ddof=1) / np.sqrt(k), (p, g[:, j])
        assert abs(d.mean()) <= 3.0 * se_d + 0.02 * abs(mean_g), (p, d.mean(), se_d, mean_g)


def test_edc_loss_absorption_gradient_matches_seed_averaged_central_differences():
    """The inverse problem as configured: the Schroeder-EDC dB loss on the
    8-material shoebox at 1e6 rays per band, materials with refraction, the
    gradient with respect to absorption through the autograd Function
    (absorption enters both the survival factor -- pathwise -- and the
    reflect / refract choice -- score terms).  With common random numbers a
    central difference (step 1e-3) of a render whose random choices flip is
    itself a noisy estimate of the derivative, so 16 seeds each give an
    adjoint gradient and a difference quotient of the full loss, compared
    in the mean."""
    torch, w, kw, tr, tgt = _seed_fd_setup()
    from ear_gb300.autograd import edc_loss, materials_from, render_materials

    spec = np.full((8, 3), 0.5)
    a0, r0 = np.full((8, 3), 0.2), np.full((8, 3), 0.05)
    step = 1e-3
    params = [(1, 0), (4, 1), (6, 2)]
    seeds = list(range(11, 27))

    def loss_at(a, seed):
        tr.set_materials(materials_from(a, r0, spec))
        h = tr.render(w.source, w.recorders, exact=True, **dict(kw, seed=seed)).hist
        return float(edc_loss(torch.from_numpy(np.asarray(h)).cuda(), tgt))

    grads, fds = [], []
    for seed in seeds:
        at = torch.tensor(a0, dtype=torch.float64, requires_grad=True)
        rt = torch.tensor(r0, dtype=torch.float64, requires_grad=True)
        hist = render_materials(at, rt, tr, w.source, w.recorders, spec, **dict(kw, seed=seed))
        edc_loss(hist, tgt).backward()
        grads.append([float(at.grad[m, b]) for m, b in params])
        f = []
        for m, b in params:
            up, dn = a0.copy(), a0.copy()
            up[m, b] += step
            dn[m, b] -= step
            f.append((loss_at(up, seed) - loss_at(dn, seed)) / (2 * step))
        fds.append(f)
    tr.close()
    _assert_seed_mean_agrees(np.array(grads), np.array(fds), params, len(seeds))


def test_edc_loss_refraction_gradient_matches_seed_averaged_central_differences():
    """The refraction half of the inverse problem.  Refraction enters only
    the reflect / refract choice, so its gradient is carried entirely by the
    estimator's score terms, which differentiate the loss's linearisation
    sum(dL/dh * h): for a loss nonlinear in h (the dB of sparsely sampled
    late energies) the expected chain-rule product and the derivative of
    the expected loss differ at O(1/N), far beyond the statistical bound
    here, so the check takes dL/dh of the EDC loss at an independent render
    (seed 98) and compares, over 16 seeds at 1e6 rays, the adjoint of that
    upstream gradient with central differences (step 1e-3, common random
    numbers) of sum(dL/dh * h) -- for absorption and refraction alike."""
    torch, w, kw, tr, tgt = _seed_fd_setup()
    from ear_gb300.autograd import edc_loss, materials_from

    spec = np.full((8, 3), 0.5)
    a0, r0 = np.full((8, 3), 0.2), np.full((8, 3), 0.05)
    tr.set_materials(materials_from(a0, r0, spec))
    h98 = torch.from_numpy(np.asarray(
        tr.render(w.source, w.recorders, exact=True, **dict(kw, seed=98)).hist)).cuda()
    h98.requires_grad_(True)
    edc_loss(h98, tgt).backward()
    g_up = h98.grad.float().contiguous()
    g64 = g_up.double().cpu().numpy()
    step = 1e-3
    params = [("r", 2, 1), ("r", 5, 2), ("a", 1, 0)]
    seeds = list(range(11, 27))

    def lin_at(a, r, seed):
        tr.set_materials(materials_from(a, r, spec))
        h = tr.render(w.source, w.recorders, exact=True, **dict(kw, seed=seed)).hist
        return float((np.asarray(h, np.float64) * g64).sum())

    grads, fds = [], []
    for seed in seeds:
        tr.set_materials(materials_from(a0, r0, spec))
        fwd = tr.render(w.source, w.recorders, exact=True, **dict(kw, seed=seed))
        g, _ = tr.render_adjoint(w.source, w.recorders, g_up, first=fwd.first_sample,
                                 last=fwd.last_sample, raw_first=fwd.raw_first_sample,
                                 raw_last=fwd.raw_last_sample, exact=True, **dict(kw, seed=seed))
        grads.append([float(g[m, b, 0 if which == "a" else 1]) for which, m, b in params])
        f = []
        for which, m, b in params:
            ua, ur, da, dr = a0.copy(), r0.copy(), a0.copy(), r0.copy()
            (ua if which == "a" else ur)[m, b] += step
            (da if which == "a" else dr)[m, b] -= step
            f.append((lin_at(ua, ur, seed) - lin_at(da, dr, seed)) / (2 * step))
        fds.append(f)
    tr.close()
    _assert_seed_mean_agrees(np.array(grads), np.array(fds), params, len(seeds))

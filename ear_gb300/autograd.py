"""Differentiable rendering: material coefficients -> impulse responses.

``render_materials(absorption, refraction, ...)`` is a
``torch.autograd.Function``: the forward pass is ``ear_render`` (exact
kernels, fixed seed, so every evaluation re-uses the same random numbers),
the backward pass is the path-replay adjoint ``ear_render_adjoint``, which
re-traces the same paths instead of storing them.  Materials are
parameterised per band by absorption a and refraction r (reflection =
1 - a - r); specularity is held fixed.  ``edc_loss`` is the Schroeder-EDC
objective of the inverse problem (squared dB differences, FP64).
"""
from __future__ import annotations

from typing import Sequence

import numpy as np
import torch

from .post import edc_db_torch
from .scene import Material, Recorder, Source, Tracer


def materials_from(absorption, refraction, specularity) -> list:
    a = np.asarray(absorption, np.float64)
    r = np.asarray(refraction, np.float64)
    sp = np.asarray(specularity, np.float64)
    return [Material(reflection=tuple((1.0 - a[i] - r[i]).tolist()), refraction=tuple(r[i].tolist()),
                     specularity=tuple(sp[i].tolist()), name=f"m{i}") for i in range(len(a))]


class _Render(torch.autograd.Function):
    @staticmethod
    def forward(ctx, absorption, refraction, tracer, source, recorders, specularity, kw):
        mats = materials_from(absorption.detach().cpu().numpy(), refraction.detach().cpu().numpy(),
                              specularity)
        tracer.set_materials(mats)
        kw = dict(kw)
        kw.setdefault("exact", True)
        res = tracer.render(source, recorders, **kw)
        ctx.tracer, ctx.source, ctx.recorders, ctx.kw, ctx.mats = tracer, source, recorders, kw, mats
        ctx.book = (res.first_sample, res.last_sample, res.raw_first_sample, res.raw_last_sample)
        ctx.like = absorption
        dev = absorption.device if absorption.is_cuda else torch.device("cuda")
        return torch.from_numpy(np.asarray(res.hist)).to(dev)

    @staticmethod
    def backward(ctx, grad_hist):
        ctx.tracer.set_materials(ctx.mats)
        first, last, raw_first, raw_last = ctx.book
        kw = dict(ctx.kw)
        g, _ = ctx.tracer.render_adjoint(ctx.source, ctx.recorders, grad_hist.float().contiguous(),
                                         first=first, last=last, raw_first=raw_first,
                                         raw_last=raw_last, **kw)
        gt = torch.from_numpy(g).to(dtype=ctx.like.dtype, device=ctx.like.device)
        return gt[..., 0], gt[..., 1], None, None, None, None, None


def render_materials(absorption: torch.Tensor, refraction: torch.Tensor, tracer: Tracer,
                     source: Source, recorders: Sequence[Recorder], specularity, **kw):
    """(tracks, 3, num_bins) impulse responses, differentiable w.r.t. the
    (materials, 3) absorption and refraction tensors."""
    return _Render.apply(absorption, refraction, tracer, source, list(recorders),
                         np.asarray(specularity), kw)


def edc_loss(hist: torch.Tensor, target_edc_db: torch.Tensor, floor_db: float = -60.0,
             track: int = 0) -> torch.Tensor:
    """sum over bands of || EDC_dB(h_band) - target ||^2 over the bins where
    the target is above ``floor_db`` (EDC in FP64)."""
    e = edc_db_torch(hist[track])  # (3, bins)
    mask = target_edc_db > floor_db
    d = torch.where(mask, e - target_edc_db, torch.zeros_like(e))
    return (d * d).sum()

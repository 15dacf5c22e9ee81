"""torch.autograd bindings of the synchrotron spectrum (thin layer over the C ABI).

    import torch
    from ragnar_gb300 import torch_ext as rt

    plan = rt.spectrum_plan(bins, B0=1.0, g_syn=1.0, e_syn_at_g_syn=1.0)   # smooth table
    S = rt.synchrotron_spectrum(plan, w, ux, uy, uz, bx, by, bz)          # [nbins]
    loss = rt.log_mse(S, S_target)
    loss.backward()                                                        # w.grad, ux.grad, ...

The forward is the fused kernel (rg_spectrum_run); the backward is the
hand-written adjoint kernel (rg_spectrum_adjoint), which recomputes e_peak
instead of storing it.  With the smooth table (the default here) the derivative
uses F'(x) = F(x)/x - x K_{5/3}(x).  All tensors are float32 on one CUDA device.
"""

from __future__ import annotations

import numpy as np
import torch

from . import capi


def spectrum_plan(bins, B0: float = 1.0, g_syn: float = 1.0, e_syn_at_g_syn: float = 1.0,
                  smooth: bool = True) -> capi.SpectrumPlan:
    """Prepared spectrum over host photon energies `bins` (numpy/list/tensor)."""
    if isinstance(bins, torch.Tensor):
        bins = bins.detach().cpu().numpy()
    mode = capi.RG_TABLE_SMOOTH if smooth else capi.RG_TABLE_REFERENCE
    return capi.SpectrumPlan(np.asarray(bins, np.float32), B0, g_syn, e_syn_at_g_syn, mode)


def dist_plan(bins, g_syn: float = 1.0, e_syn_at_g_syn: float = 1.0, log_spaced: bool = True,
              smooth: bool = True) -> capi.DistPlan:
    if isinstance(bins, torch.Tensor):
        bins = bins.detach().cpu().numpy()
    mode = capi.RG_TABLE_SMOOTH if smooth else capi.RG_TABLE_REFERENCE
    return capi.DistPlan(np.asarray(bins, np.float32), g_syn, e_syn_at_g_syn, log_spaced, mode)


def _check(t: torch.Tensor | None, name: str, dev) -> None:
    if t is None:
        return
    if t.dtype != torch.float32 or not t.is_cuda or not t.is_contiguous():
        raise ValueError(f"{name} must be a contiguous float32 CUDA tensor")
    if dev is not None and t.device != dev:
        raise ValueError(f"{name} is on {t.device}, expected {dev}")


def _stream(dev) -> int:
    return torch.cuda.current_stream(dev).cuda_stream


class _Spectrum(torch.autograd.Function):
    @staticmethod
    def forward(ctx, plan, w, ux, uy, uz, bx, by, bz, ex, ey, ez):  # noqa: PLR0913
        dev = ux.device
        for name, t in (("w", w), ("ux", ux), ("uy", uy), ("uz", uz), ("bx", bx), ("by", by),
                        ("bz", bz), ("ex", ex), ("ey", ey), ("ez", ez)):
            _check(t, name, dev)
        e = None if ex is None else [ex, ey, ez]
        prt = capi.particles([ux, uy, uz], b=[bx, by, bz], e=e, w=w, n=ux.numel())
        out = torch.empty(plan.nbins, device=dev, dtype=torch.float32)
        # on cell-moment plans the forward records each particle's table placement (8 bytes per
        # particle), which the backward then reads instead of placing the particle again
        place = None
        if plan.placement_supported():
            place = torch.empty(2 * ux.numel(), device=dev, dtype=torch.int32)
            plan.run_placed(prt, out, place, _stream(dev))
        else:
            plan.run(prt, out, _stream(dev))
        ctx.plan = plan
        ctx.save_for_backward(w, ux, uy, uz, bx, by, bz, ex, ey, ez, place)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        w, ux, uy, uz, bx, by, bz, ex, ey, ez, place = ctx.saved_tensors
        dev = ux.device
        need_w, need_u = ctx.needs_input_grad[1], any(ctx.needs_input_grad[2:5])
        gw = torch.empty_like(ux) if (need_w and w is not None) else None
        gu = [torch.empty_like(ux) if ctx.needs_input_grad[2 + d] else None for d in range(3)]
        if gw is None and not need_u:
            return (None,) * 11
        e = None if ex is None else [ex, ey, ez]
        prt = capi.particles([ux, uy, uz], b=[bx, by, bz], e=e, w=w, n=ux.numel())
        if place is not None:
            ctx.plan.adjoint_placed(prt, place, grad_out.contiguous().float(), gw, gu, _stream(dev))
        else:
            ctx.plan.adjoint(prt, grad_out.contiguous().float(), gw, gu, _stream(dev))
        return (None, gw, gu[0], gu[1], gu[2], None, None, None, None, None, None)


def synchrotron_spectrum(plan: capi.SpectrumPlan, w, ux, uy, uz, bx, by, bz, ex=None, ey=None, ez=None):
    """Differentiable particle spectrum S[b] = e_b sum_p w_p chiR_p F(e_b / e_peak_p).

    Gradients flow to w and ux, uy, uz.  `w` may be None (unit weights)."""
    return _Spectrum.apply(plan, w, ux, uy, uz, bx, by, bz, ex, ey, ez)


class _FromDist(torch.autograd.Function):
    @staticmethod
    def forward(ctx, plan, gbeta, f):
        dev = f.device
        _check(gbeta, "gbeta", dev)
        _check(f, "f", dev)
        out = torch.empty(plan.nbins, device=dev, dtype=torch.float32)
        plan.run_dist(gbeta, f, out, _stream(dev))
        ctx.plan = plan
        ctx.save_for_backward(gbeta, f)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        gbeta, f = ctx.saved_tensors
        gf = torch.empty_like(f)
        ctx.plan.adjoint_dist(gbeta, f, grad_out.contiguous().float(), gf, _stream(f.device))
        return None, None, gf


def synchrotron_from_dist(plan: capi.DistPlan, gbeta, f):
    """Differentiable spectrum of one tabulated distribution; gradients flow to f."""
    return _FromDist.apply(plan, gbeta, f)


def log_mse(S, S_target, floor: float = 1e-12):
    """mean of (log S - log S_target)^2 over the bins where both spectra exceed
    `floor` times their peak (bins with a vanishing spectrum are left out: their
    1/S weight would overflow and carries no information)."""
    m = (S > floor * S.detach().max()) & (S_target > floor * S_target.max())
    d = torch.log(torch.where(m, S, torch.ones_like(S))) - torch.log(
        torch.where(m, S_target, torch.ones_like(S_target)))
    return (d * d * m).sum() / m.sum().clamp(min=1)


def fromdist_plan(gbeta, bins, g_syn: float = 1.0, e_syn_at_g_syn: float = 1.0, log_spaced: bool = True,
                  max_dist: int = 1024, smooth: bool = True, split_products: int = 6) -> capi.FromDistPlan:
    """Tensor-core plan for many distributions on the same gamma bins."""
    to_np = lambda a: a.detach().cpu().numpy() if isinstance(a, torch.Tensor) else np.asarray(a)  # noqa: E731
    mode = capi.RG_TABLE_SMOOTH if smooth else capi.RG_TABLE_REFERENCE
    return capi.FromDistPlan(to_np(gbeta), log_spaced, to_np(bins), g_syn, e_syn_at_g_syn, max_dist, mode,
                             split_products)


class _FromDistBatched(torch.autograd.Function):
    @staticmethod
    def forward(ctx, plan, f):
        _check(f, "f", f.device)
        out = torch.empty((f.shape[0], plan.nbins), device=f.device, dtype=torch.float32)
        plan.run(f, out, _stream(f.device))
        ctx.plan = plan
        return out

    @staticmethod
    def backward(ctx, grad_out):
        g = grad_out.contiguous().float()
        gf = torch.empty((g.shape[0], ctx.plan.ng), device=g.device, dtype=torch.float32)
        ctx.plan.adjoint(g, gf, _stream(g.device))
        return None, gf


def synchrotron_from_dist_batched(plan: capi.FromDistPlan, f):
    """Spectra [ndist, nbins] of distributions f [ndist, ng]: BF16 split-precision
    tensor-core GEMM forward, transpose GEMM adjoint."""
    return _FromDistBatched.apply(plan, f)

"""The differentiable path: the smooth F table built on the GPU, the smooth-mode
forward, and the adjoint behind torch.autograd, checked against the FP64 oracle
(its own table from std::cyl_bessel_k, its analytic gradient) and against FP64
central finite differences (h = 1e-6 relative) of a log-space loss on 64
randomly chosen particles.  Log-uniform photon bins give a plan its own smooth
table aligned to the bins; both ways of summing run on it: the fused kernels
(every particle x bin pair) and the cell moments (forward: four moments per
table cell; adjoint: one cubic per cell)."""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from helpers import SPECTRUM_RTOL, max_rel, particles

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
capi = pytest.importorskip("ragnar_gb300.capi")
rt = pytest.importorskip("ragnar_gb300.torch_ext")


@pytest.fixture(scope="module")
def smooth(gpu):
    nseg = ctypes.c_int32()
    lnx, dln = ctypes.c_double(), ctypes.c_double()
    capi.check(capi.lib().rg_smooth_table(None, ctypes.byref(nseg), ctypes.byref(lnx), ctypes.byref(dln)))
    coef = np.empty((nseg.value, 4), np.float32)
    capi.check(capi.lib().rg_smooth_table(coef.ctypes.data, None, None, None))
    return coef, lnx.value, dln.value


def test_smooth_table_matches_independent_oracle(oracle_lib, smooth):
    coef, lnx, dln = smooth
    ref = oracle_lib.smooth_coefficients(coef.shape[0])
    assert abs(lnx - np.log(oracle_lib.SMOOTH_XMIN)) < 1e-15
    # values and slopes of exact F from two independent FP64 quadratures, rounded to
    # float; segments where F has fallen below float's normal range compare absolutely
    scale = np.abs(ref[:, 0:1]) + np.abs(ref[:, 1:2])
    big = scale[:, 0] > 1e-30
    assert np.max(np.abs(coef[big] - ref[big]) / scale[big]) < 3e-7
    assert np.max(np.abs(coef[~big] - ref[~big])) < 1e-36


ALGOS = [pytest.param(1, id="direct"), pytest.param(2, id="moments")]


def plan_table(plan):
    """(coef, xmin, xmax) of the smooth table a plan evaluates, for the oracle."""
    coef, lnx, dln = plan.smooth_table()
    return coef, float(np.exp(lnx)), float(np.exp(lnx + coef.shape[0] * dln))


def test_plan_table_matches_independent_oracle(gpu, oracle_lib):
    """A plan's own (bin-aligned) table against the oracle's FP64 Hermite coefficients
    on the same geometry; bins that are not log-uniform keep the device-wide table."""
    plan = rt.spectrum_plan(oracle_lib.logspace(0.01, 1e7, 512))
    coef, xmin, xmax = plan_table(plan)
    assert coef.shape[0] != 2048 and xmin <= 1e-6 * (1 + 1e-12) and xmax >= 100.0 * (1 - 1e-12)
    ref = oracle_lib.smooth_coefficients(coef.shape[0], xmin, xmax)
    scale = np.abs(ref[:, 0:1]) + np.abs(ref[:, 1:2])
    big = scale[:, 0] > 1e-30
    assert np.max(np.abs(coef[big] - ref[big]) / scale[big]) < 3e-7
    uneven = rt.spectrum_plan(np.array([0.1, 0.3, 2.0, 50.0, 51.0], np.float32))
    assert uneven.smooth_table()[0].shape[0] == 2048
    assert uneven.algorithm(1) == capi.RG_ALGO_DIRECT
    assert plan.algorithm(1) == capi.RG_ALGO_MOMENTS


def _device(P, dev):
    return {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in P.items()}


@pytest.mark.parametrize("algo", ALGOS)
@pytest.mark.parametrize("nbins,lo,hi", [(200, 0.01, 1e7), (512, 0.01, 1e7), (77, 1e-3, 1e5), (1500, 1e-4, 1e9)])
def test_smooth_forward(gpu, oracle_lib, nbins, lo, hi, algo):
    P = particles(20000, seed=nbins, bfield="iso", weights=True)
    bins = oracle_lib.logspace(lo, hi, nbins)
    T = _device(P, gpu)
    plan = rt.spectrum_plan(bins)
    plan.set_algorithm(algo)
    S = rt.synchrotron_spectrum(plan, T["w"], T["ux"], T["uy"], T["uz"], T["bx"], T["by"], T["bz"])
    coef, xmin, xmax = plan_table(plan)
    truth = oracle_lib.sync_smooth_f64(P, bins, 1.0, 1.0, 1.0, coef, xmin, xmax)
    assert max_rel(S.cpu().numpy(), truth) <= SPECTRUM_RTOL


def _log_loss_np(S, St, floor=1e-12):
    # the loss of ragnar_gb300.torch_ext.log_mse: bins above floor x peak in both spectra
    m = (S > floor * S.max()) & (St > floor * St.max())
    return np.sum((np.log(S[m]) - np.log(St[m])) ** 2) / m.sum(), m


@pytest.mark.parametrize("algo", ALGOS)
def test_adjoint_vs_fp64_gradient_and_finite_differences(gpu, oracle_lib, algo):
    n, nbins = 4000, 512
    P = particles(n, seed=21, bfield="iso", weights=True)
    Pt = particles(n, seed=22, bfield="iso", weights=True, index=-2.5, umax=300.0)
    bins = oracle_lib.logspace(0.01, 1e7, nbins)
    plan = rt.spectrum_plan(bins)
    plan.set_algorithm(algo)
    coef, xmin, xmax = plan_table(plan)
    S64 = oracle_lib.sync_smooth_f64(P, bins, 1.0, 1.0, 1.0, coef, xmin, xmax)
    St = oracle_lib.sync_smooth_f64(Pt, bins, 1.0, 1.0, 1.0, coef, xmin, xmax)
    L0, m = _log_loss_np(S64, St)
    M = m.sum()
    gS = np.zeros(nbins)
    gS[m] = 2.0 * (np.log(S64[m]) - np.log(St[m])) / (M * S64[m])

    # GPU adjoint driven by the same dL/dS
    T = _device(P, gpu)
    prt = capi.particles([T["ux"], T["uy"], T["uz"]], b=[T["bx"], T["by"], T["bz"]], w=T["w"])
    gw = torch.empty(n, device=gpu)
    gu = [torch.empty(n, device=gpu) for _ in range(3)]
    plan.adjoint(prt, torch.from_numpy(gS.astype(np.float32)).to(gpu), gw, gu)
    plan.check()
    g_gpu = np.stack([gw.cpu().numpy()] + [g.cpu().numpy() for g in gu]).astype(np.float64)

    # FP64 analytic gradient of the same function
    gw64, gu64 = oracle_lib.sync_smooth_grad_f64(P, bins, 1.0, 1.0, 1.0, coef, gS, xmin, xmax)
    g64 = np.vstack([gw64[None], gu64])
    scale = np.max(np.abs(g64), axis=1, keepdims=True)
    assert np.max(np.abs(g_gpu - g64) / scale) < 1e-4

    # FP64 central finite differences of the loss on 64 random particles.  The mask is
    # held fixed (log_mse takes it from the detached spectrum), and the difference
    # L(x+h) - L(x-h) = sum (lS+ - lS-)(lS+ + lS- - 2 lS_t) / M is formed from the
    # single-particle spectra, so no O(1) loss values are subtracted from each other.
    rng = np.random.default_rng(5)
    keys = ("ux", "uy", "uz", "bx", "by", "bz", "w")
    lt = np.log(St[m])
    worst = 0.0
    for p in rng.choice(n, 64, replace=False):
        one = {k: P[k][p:p + 1].astype(np.float64) for k in keys}
        s_p = oracle_lib.sync_smooth_f64(one, bins, 1.0, 1.0, 1.0, coef, xmin, xmax)
        rest = S64 - s_p
        for c, key in enumerate(("w", "ux", "uy", "uz")):
            x0 = one[key][0]
            h = 1e-6 * abs(x0) if x0 != 0 else 1e-9
            s_pm = []
            for sgn in (1.0, -1.0):
                q = {k: v.copy() for k, v in one.items()}
                q[key][0] = x0 + sgn * h
                s_pm.append(oracle_lib.sync_smooth_f64(q, bins, 1.0, 1.0, 1.0, coef, xmin, xmax))
            Sp, Sm = rest + s_pm[0], rest + s_pm[1]
            dlog = np.log1p((s_pm[0] - s_pm[1])[m] / Sm[m])
            fd = np.sum(dlog * (np.log(Sp[m]) + np.log(Sm[m]) - 2.0 * lt)) / M / (2 * h)
            ref = max(abs(fd), 1e-3 * scale[c, 0])
            worst = max(worst, abs(g_gpu[c, p] - fd) / ref)
            # the FP64 gradient itself against FD: the table is C1 (piecewise cubic), so a
            # central difference straddling a segment joint is off by O(h |jump of F''|)
            assert abs(g64[c, p] - fd) <= 1e-5 * ref + 1e-12, (p, key)
    assert worst < 1e-4, worst


@pytest.mark.parametrize("algo", ALGOS)
def test_autograd_end_to_end(gpu, oracle_lib, algo):
    n, nbins = 3000, 256
    P = particles(n, seed=31, bfield="iso", weights=True, efield=True)
    bins = oracle_lib.logspace(0.01, 1e6, nbins)
    T = _device(P, gpu)
    for k in ("w", "ux", "uy", "uz"):
        T[k].requires_grad_(True)
    plan = rt.spectrum_plan(bins)
    plan.set_algorithm(algo)
    coef, xmin, xmax = plan_table(plan)
    S = rt.synchrotron_spectrum(plan, T["w"], T["ux"], T["uy"], T["uz"], T["bx"], T["by"], T["bz"],
                                T["ex"], T["ey"], T["ez"])
    target = S.detach() * torch.linspace(0.5, 1.5, nbins, device=gpu)
    loss = rt.log_mse(S, target)
    loss.backward()
    S64 = oracle_lib.sync_smooth_f64(P, bins, 1.0, 1.0, 1.0, coef, xmin, xmax)
    St = S64 * np.linspace(0.5, 1.5, nbins, dtype=np.float32).astype(np.float64)
    _, m = _log_loss_np(S64, St)
    gS = np.zeros(nbins)
    gS[m] = 2.0 * (np.log(S64[m]) - np.log(St[m])) / (m.sum() * S64[m])
    gw64, gu64 = oracle_lib.sync_smooth_grad_f64(P, bins, 1.0, 1.0, 1.0, coef, gS, xmin, xmax)
    for got, want in [(T["w"].grad, gw64)] + [(T[k].grad, gu64[i]) for i, k in enumerate(("ux", "uy", "uz"))]:
        g = got.cpu().numpy()
        assert np.max(np.abs(g - want)) / np.max(np.abs(want)) < 1e-3


def test_placed_forward_and_adjoint_match_unplaced(gpu, oracle_lib):
    """rg_spectrum_run_placed records each particle's table placement; the adjoint that reads
    it equals the one that places the particles again bit for bit, and particles that add
    nothing (zero field, huge energy) are recorded as such.  Plans that do not run cell
    moments on an aligned smooth table refuse both calls."""
    n, nbins = 20000, 200
    P = particles(n, seed=53, bfield="iso", weights=True)
    P["bx"][:50] = 0.0
    P["by"][:50] = 0.0
    P["bz"][:50] = 0.0  # W = 0: no emission
    P["ux"][50:60] = 3e8  # e_peak far above the table
    T = _device(P, gpu)
    prt = capi.particles([T["ux"], T["uy"], T["uz"]], b=[T["bx"], T["by"], T["bz"]], w=T["w"])
    plan = rt.spectrum_plan(oracle_lib.logspace(0.01, 1e7, nbins))
    assert plan.placement_supported()
    S0, S1 = torch.empty(nbins, device=gpu), torch.empty(nbins, device=gpu)
    place = torch.full((2 * n,), -7, dtype=torch.int32, device=gpu)
    plan.run(prt, S0)
    plan.run_placed(prt, S1, place)
    a64, b64 = S1.double(), S0.double()
    assert bool(((a64 - b64).abs() <= 1.2e-7 * b64.abs().clamp(min=1e-300)).all())
    rec = place.view(n, 2).cpu().numpy().view(np.uint32)
    assert np.all(rec[:50, 0] == 0xFFFFFFFF) and np.all(rec[:50, 1] == 0)
    assert not np.any(place.cpu().numpy() == -7)  # every particle written
    gS = torch.rand(nbins, device=gpu)
    g0 = [torch.empty(n, device=gpu) for _ in range(4)]
    g1 = [torch.empty(n, device=gpu) for _ in range(4)]
    plan.adjoint(prt, gS, g0[0], g0[1:])
    plan.adjoint_placed(prt, place, gS, g1[0], g1[1:])
    plan.check()
    for a, b in zip(g0, g1):
        assert torch.equal(a, b)
    assert torch.all(g1[0][:50] == 0)
    ref = capi.SpectrumPlan(oracle_lib.logspace(0.01, 1e7, nbins), 1.0, 1.0, 1.0)
    assert not ref.placement_supported()
    with pytest.raises(capi.RgError):
        ref.run_placed(prt, S1, place)
    with pytest.raises(capi.RgError):
        ref.adjoint_placed(prt, place, gS, g1[0])
    with pytest.raises(capi.RgError):
        plan.run_placed(prt, S1, None)


@pytest.mark.parametrize("algo", ALGOS)
def test_batched_adjoint_matches_per_segment(gpu, oracle_lib, algo):
    P = particles(9000, seed=41, bfield="iso", weights=True)
    bins = oracle_lib.logspace(0.01, 1e7, 128)
    T = _device(P, gpu)
    prt = capi.particles([T["ux"], T["uy"], T["uz"]], b=[T["bx"], T["by"], T["bz"]], w=T["w"])
    plan = rt.spectrum_plan(bins)
    plan.set_algorithm(algo)
    offs = torch.tensor([0, 2000, 2000, 9000], dtype=torch.int64, device=gpu)
    plan.reserve(3)
    gS = torch.rand((3, 128), device=gpu)
    gw = torch.empty(9000, device=gpu)
    plan.adjoint_batched(prt, offs, 3, gS, gw)
    plan.check()
    for s, (a, b) in enumerate([(0, 2000), (2000, 9000)]):
        sub = capi.particles([T["ux"][a:b], T["uy"][a:b], T["uz"][a:b]],
                             b=[T["bx"][a:b], T["by"][a:b], T["bz"][a:b]], w=T["w"][a:b])
        g1 = torch.empty(b - a, device=gpu)
        plan.adjoint(sub, gS[0 if s == 0 else 2].contiguous(), g1)
        np.testing.assert_allclose(gw[a:b].cpu().numpy(), g1.cpu().numpy(), rtol=1e-6, atol=1e-12)


def test_dist_adjoint(gpu, oracle_lib, smooth):
    coef, lnx, dln = smooth
    gb = oracle_lib.logspace(1.0, 1e5, 300)
    f = (gb.astype(np.float64) ** -2.2).astype(np.float32)
    bins = oracle_lib.logspace(0.01, 1e11, 400)
    plan = rt.dist_plan(bins, log_spaced=True)
    g_t = torch.from_numpy(gb).to(gpu)
    f_t = torch.from_numpy(f).to(gpu).requires_grad_(True)
    S = rt.synchrotron_from_dist(plan, g_t, f_t)
    w = torch.rand(400, device=gpu)
    (S * w).sum().backward()
    # FP64: K[b, g] = e_b gbeta_g F(e_b / gbeta_g^2) with the smooth table
    x = np.log(bins.astype(np.float64))[:, None] - 2.0 * np.log(gb.astype(np.float64))[None, :]
    t = (x - lnx) / dln
    j = np.floor(t).astype(np.int64)
    ok = (t >= 0) & (t < coef.shape[0])
    jj = np.clip(j, 0, coef.shape[0] - 1)
    tau = t - jj
    c = coef.astype(np.float64)[jj]
    F = np.where(ok, c[..., 0] + tau * (c[..., 1] + tau * (c[..., 2] + tau * c[..., 3])), 0.0)
    K = bins.astype(np.float64)[:, None] * gb.astype(np.float64)[None, :] * F
    S64 = K @ f.astype(np.float64)
    assert max_rel(S.detach().cpu().numpy(), S64) <= SPECTRUM_RTOL
    gf64 = K.T @ w.cpu().numpy().astype(np.float64)
    gf = f_t.grad.cpu().numpy()
    assert np.max(np.abs(gf - gf64)) / np.max(np.abs(gf64)) < 1e-5


@pytest.mark.parametrize("algo", ALGOS)
def test_smooth_host_streaming_matches_device(gpu, oracle_lib, algo):
    """Host-resident particles of several staging chunks through a smooth plan (its moments
    accumulate over the chunks) match the same particles resident on the device and the
    FP64 oracle on the plan's table."""
    n = (1 << 22) + 3001
    P = particles(n, seed=61, bfield="iso", weights=True)
    bins = oracle_lib.logspace(0.01, 1e7, 256)
    plan = rt.spectrum_plan(bins)
    plan.set_algorithm(algo)
    H = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in P.items()}
    hprt = capi.host_particles([H["ux"], H["uy"], H["uz"]], b=[H["bx"], H["by"], H["bz"]], w=H["w"], n=n)
    out = torch.empty(256, device=gpu)
    plan.run_host(hprt, out)
    T = _device(P, gpu)
    prt = capi.particles([T["ux"], T["uy"], T["uz"]], b=[T["bx"], T["by"], T["bz"]], w=T["w"])
    dev = torch.empty(256, device=gpu)
    plan.run(prt, dev)
    plan.check()
    assert max_rel(out.cpu().numpy(), dev.cpu().numpy()) <= 1e-6
    coef, xmin, xmax = plan_table(plan)
    sub = {k: v[:200000] for k, v in P.items()}
    T2 = _device(sub, gpu)
    prt2 = capi.particles([T2["ux"], T2["uy"], T2["uz"]], b=[T2["bx"], T2["by"], T2["bz"]], w=T2["w"])
    plan.run(prt2, dev)
    plan.check()
    truth = oracle_lib.sync_smooth_f64(sub, bins, 1.0, 1.0, 1.0, coef, xmin, xmax)
    assert max_rel(dev.cpu().numpy(), truth) <= SPECTRUM_RTOL

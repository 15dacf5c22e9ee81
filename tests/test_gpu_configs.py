"""Two benchmark configurations checked against the FP64 oracle at their stated sizes.

* The small CPU-runnable configuration: SynchrotronSpectrum_3D of 1e6 particles
  (|u| ~ u^-2 on [1, 100] by inverse CDF, isotropic directions, unit weights,
  B = (0, 0, 1)) into 200 log photon bins 0.01..1e7 mec2, and
  Particles.energyDistribution of the same particles into 200 log bins
  1e-2..1e3, through the drop-in module as the reference's own test drives it
  (tests/synchrotron.py:62-104: power-law U1 by inverse CDF, fromArrays,
  energyDistribution, SynchrotronSpectrum_3D).
* The differentiation configuration: 1e7 particles of the same kind x 512 log
  bins 0.01..1e7, loss = log-space MSE to a target made from the same setup at
  index -2.5 with an exp(-gamma/300) cutoff; the autograd gradient with respect
  to the weights and four-velocities against the FP64 oracle's full analytic
  gradient (every particle) and against FP64 central finite differences
  (h = 1e-6 relative) on 64 randomly chosen particles.
"""

from __future__ import annotations

import numpy as np
import pytest

from helpers import SPECTRUM_RTOL, isotropic, max_rel, powerlaw

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
rg = pytest.importorskip("ragnar_gb300")
capi = pytest.importorskip("ragnar_gb300.capi")
rt = pytest.importorskip("ragnar_gb300.torch_ext")


def config1_particles(n, seed=0, index=-2.0, umax=100.0, gcut=None):
    rng = np.random.default_rng(seed)
    if gcut is None:
        umag = powerlaw(rng, n, 1.0, umax, index)
    else:  # power law times exp(-gamma / gcut), by rejection
        umag = np.empty(0)
        while umag.size < n:
            m = 2 * (n - umag.size) + 1024
            u = powerlaw(rng, m, 1.0, umax, index)
            umag = np.concatenate([umag, u[rng.random(m) < np.exp(-np.sqrt(1.0 + u * u) / gcut)]])
        umag = umag[:n]
    u = isotropic(rng, n, umag)
    z = np.zeros(n, np.float32)
    return {"ux": u[0], "uy": u[1], "uz": u[2], "bx": z, "by": z.copy(), "bz": np.ones(n, np.float32)}


def test_config1_spectrum_and_histogram_at_full_size(gpu, oracle_lib):
    n = 1_000_000
    P = config1_particles(n, seed=0)
    rg.Initialize()
    prtls = rg.Particles_3D("pairs")
    prtls.fromArrays({"U1": P["ux"], "U2": P["uy"], "U3": P["uz"], "B3": P["bz"]})

    bins = rg.Logbins(0.01, 1e7, 200, rg.EnergyUnits.mec2)
    S = rg.SynchrotronSpectrum_3D(prtls, bins, 1, 1, 1).as_array()
    truth = oracle_lib.sync_spectrum_f64(P, bins.as_array(), 1.0, 1.0, 1.0, oracle_lib.tabulate_ffunc())
    assert max_rel(S, truth) <= SPECTRUM_RTOL
    assert np.array_equal(S == 0, truth == 0)

    ebins = rg.Logbins(1e-2, 1e3, 200)
    dist = prtls.energyDistribution(ebins)
    _, h64, counts = oracle_lib.energy_distribution(P["ux"], P["uy"], P["uz"], ebins.as_array(), True, True)
    F = dist.F().as_array()
    m = h64 > 0
    assert np.max(np.abs(F[m] - h64[m]) / h64[m]) < 1e-5
    assert np.all(F[~m] == 0)
    # integer counts bit-exact through the C ABI
    T = [torch.from_numpy(P[k]).to(gpu) for k in ("ux", "uy", "uz")]
    hist = torch.empty(200, device=gpu)
    cnt = torch.empty(200, dtype=torch.int64, device=gpu)
    eb = ebins.as_array().astype(np.float32)
    capi.check(capi.lib().rg_energy_distribution(T[0].data_ptr(), T[1].data_ptr(), T[2].data_ptr(), n,
                                                 eb.ctypes.data, 200, 1, 1, hist.data_ptr(), cnt.data_ptr(), 0))
    torch.cuda.synchronize()
    np.testing.assert_array_equal(cnt.cpu().numpy(), counts)
    assert int(counts.sum()) == n


@pytest.mark.parametrize("algo", [pytest.param(1, id="direct"), pytest.param(2, id="moments")])
def test_config4_gradient_at_full_size(gpu, oracle_lib, algo):
    n, nbins = 10_000_000, 512
    P = config1_particles(n, seed=4)
    P["w"] = np.ones(n, np.float32)
    Pt = config1_particles(2_000_000, seed=44, index=-2.5, umax=1e4, gcut=300.0)
    bins = oracle_lib.logspace(0.01, 1e7, nbins)
    plan = rt.spectrum_plan(bins)
    plan.set_algorithm(algo)
    coef, lnx, dln = plan.smooth_table()
    xmin, xmax = float(np.exp(lnx)), float(np.exp(lnx + coef.shape[0] * dln))

    T = {k: torch.from_numpy(v).to(gpu) for k, v in P.items()}
    Tt = {k: torch.from_numpy(v).to(gpu) for k, v in Pt.items()}
    with torch.no_grad():
        St = rt.synchrotron_spectrum(plan, None, Tt["ux"], Tt["uy"], Tt["uz"], Tt["bx"], Tt["by"], Tt["bz"])
    for k in ("w", "ux", "uy", "uz"):
        T[k].requires_grad_(True)
    S = rt.synchrotron_spectrum(plan, T["w"], T["ux"], T["uy"], T["uz"], T["bx"], T["by"], T["bz"])
    loss = rt.log_mse(S, St)
    loss.backward()
    plan.check()
    g_gpu = np.stack([T[k].grad.cpu().numpy() for k in ("w", "ux", "uy", "uz")]).astype(np.float64)

    # forward and full gradient in FP64 (every particle), driven by the FP64 dL/dS
    S64 = oracle_lib.sync_smooth_f64(P, bins, 1.0, 1.0, 1.0, coef, xmin, xmax)
    assert max_rel(S.detach().cpu().numpy(), S64) <= SPECTRUM_RTOL
    St_np = St.cpu().numpy().astype(np.float64)
    m = (S64 > 1e-12 * S64.max()) & (St_np > 1e-12 * St_np.max())
    M = m.sum()
    gS = np.zeros(nbins)
    gS[m] = 2.0 * (np.log(S64[m]) - np.log(St_np[m])) / (M * S64[m])
    gw64, gu64 = oracle_lib.sync_smooth_grad_f64(P, bins, 1.0, 1.0, 1.0, coef, gS, xmin, xmax)
    g64 = np.vstack([gw64[None], gu64])
    scale = np.max(np.abs(g64), axis=1, keepdims=True)
    assert np.max(np.abs(g_gpu - g64) / scale) < 1e-4

    # FP64 central finite differences on 64 random particles, formed from the
    # single-particle spectra so that no O(1) loss values cancel
    rng = np.random.default_rng(404)
    keys = ("ux", "uy", "uz", "bx", "by", "bz", "w")
    lt = np.log(St_np[m])
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
    assert worst < 1e-4, worst

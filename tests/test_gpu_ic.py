"""Inverse-Compton spectrum on the GPU (rg_ic_spectrum, ICSpectrum ic.cpp:15-46) against
the FP64 oracle and the reference build's golden outputs, with the edge cases the
kernel handles explicitly (bins above the Klein-Nishina limit, invalid IC bins,
empty inputs, more than one 512-bin slice) and the drop-in module's unit checks."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import SPECTRUM_RTOL, golden, max_rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
capi = pytest.importorskip("ragnar_gb300.capi")


def gpu_ic(gb, fp, log_spaced, es, fs, eic, dev):
    t = [torch.from_numpy(np.ascontiguousarray(a, np.float32)).to(dev) for a in (gb, fp, es, fs, eic)]
    out = torch.full((len(eic),), -1.0, device=dev)
    capi.check(capi.lib().rg_ic_spectrum(t[0].data_ptr(), t[1].data_ptr(), len(gb), int(log_spaced),
                                         t[2].data_ptr(), t[3].data_ptr(), len(es), t[4].data_ptr(), len(eic),
                                         out.data_ptr(), 0))
    torch.cuda.synchronize()
    return out.cpu().numpy()


@pytest.mark.parametrize("case", [0, 1, 2])
def test_golden_cases(gpu, oracle_lib, case):
    g = golden("ic")
    args = (g[f"case{case}_gb"], g[f"case{case}_f"], bool(g[f"case{case}_log"]), g[f"case{case}_es"],
            g[f"case{case}_fs"], g[f"case{case}_eic"])
    got = gpu_ic(*args, gpu)
    assert max_rel(got, oracle_lib.ic_spectrum_f64(*args)) <= SPECTRUM_RTOL
    # the reference's own float arithmetic is ~2e-5 from FP64 near the Klein-Nishina cutoff
    assert max_rel(got, g[f"case{case}_ref"]) <= 5e-5


@pytest.mark.parametrize("log_spaced", [True, False])
def test_random_two_slices(gpu, oracle_lib, log_spaced):
    rng = np.random.default_rng(7 + log_spaced)
    gb = oracle_lib.logspace(10.0, 1e6, 300) if log_spaced else oracle_lib.linspace(10.0, 1e6, 300)
    fp = (gb.astype(np.float64) ** -2.3 * np.exp(-gb / 3e5)).astype(np.float32)
    es = oracle_lib.logspace(1e-9, 1e-3, 150)
    fs = (rng.uniform(0.5, 1.5, 150) * es.astype(np.float64) ** -1.0).astype(np.float32)
    eic = oracle_lib.logspace(1e-3, 1e6, 700)
    got = gpu_ic(gb, fp, log_spaced, es, fs, eic, gpu)
    assert max_rel(got, oracle_lib.ic_spectrum_f64(gb, fp, log_spaced, es, fs, eic)) <= SPECTRUM_RTOL


def test_invalid_and_unreachable_bins(gpu, oracle_lib):
    gb = oracle_lib.logspace(1e3, 1e5, 64)
    fp = np.ones(64, np.float32)
    es = oracle_lib.logspace(1e-9, 1e-7, 40)
    fs = np.ones(40, np.float32)
    eic = oracle_lib.logspace(1e2, 1e6, 90)
    eic[[0, 5, 9]] = [0.0, -3.0, np.nan]
    got = gpu_ic(gb, fp, True, es, fs, eic, gpu)
    assert np.all(got[[0, 5, 9]] == 0.0)
    assert np.all(got[eic > 1e5] == 0.0)  # above every gamma bin: no pair reaches it
    good = np.isfinite(eic) & (eic > 0)
    want = oracle_lib.ic_spectrum_f64(gb, fp, True, es, fs, eic[good])
    assert max_rel(got[good], want) <= SPECTRUM_RTOL


def test_wide_and_masked_soft_photons(gpu, oracle_lib):
    """Soft photons over 39 decades in one 64-photon chunk (q from far below 1e-30 to far
    above 1: the floor on t/g and max(KN, 0) at both ends), a ragged last chunk, and masked
    photons (e_s <= 0, NaN, 1/(4 e_s) overflowing) that contribute nothing."""
    gb = oracle_lib.logspace(10.0, 1e6, 200)
    fp = (gb.astype(np.float64) ** -2.0).astype(np.float32)
    es = np.concatenate([oracle_lib.logspace(1e-36, 1e3, 64),
                         oracle_lib.logspace(1e-9, 1e-5, 64),
                         oracle_lib.logspace(1e-9, 1e-5, 40)])
    fs = np.ones(len(es), np.float32)
    eic = oracle_lib.logspace(1e-3, 1e6, 300)
    got = gpu_ic(gb, fp, True, es, fs, eic, gpu)
    assert max_rel(got, oracle_lib.ic_spectrum_f64(gb, fp, True, es, fs, eic)) <= SPECTRUM_RTOL

    bad = es.copy()
    idx = [3, 70, 130, 150]
    bad[idx] = [0.0, -1e-8, np.nan, 1e-45]  # the last: 4 e_s is subnormal, 1/(4 e_s) = inf
    keep = np.ones(len(es), bool)
    keep[idx] = False
    got = gpu_ic(gb, fp, True, bad, fs, eic, gpu)
    want = oracle_lib.ic_spectrum_f64(gb, fp, True, bad[keep], fs[keep], eic)
    assert max_rel(got, want) <= SPECTRUM_RTOL


def test_large_grid_without_setup_table(gpu, oracle_lib):
    """8192 gamma bins x 1024 IC bins: the per-call (gamma bin, IC bin) setup table would take
    134 MB, above its 64 MB cap, so the kernel computes each pair's setup per item instead."""
    gb = oracle_lib.logspace(10.0, 1e6, 8192)
    fp = (gb.astype(np.float64) ** -2.0 * np.exp(-gb / 3e5)).astype(np.float32)
    es = oracle_lib.logspace(1e-9, 1e-5, 16)
    fs = np.ones(16, np.float32)
    eic = oracle_lib.logspace(1e-3, 1e6, 1024)
    got = gpu_ic(gb, fp, True, es, fs, eic, gpu)
    assert max_rel(got, oracle_lib.ic_spectrum_f64(gb, fp, True, es, fs, eic)) <= SPECTRUM_RTOL


def test_empty_inputs(gpu):
    dev = gpu
    z = torch.zeros(4, device=dev)
    out = torch.full((4,), 7.0, device=dev)
    L = capi.lib()
    capi.check(L.rg_ic_spectrum(z.data_ptr(), z.data_ptr(), 0, 1, z.data_ptr(), z.data_ptr(), 4,
                                z.data_ptr(), 4, out.data_ptr(), 0))
    torch.cuda.synchronize()
    assert torch.all(out == 0)
    capi.check(L.rg_ic_spectrum(z.data_ptr(), z.data_ptr(), 4, 1, z.data_ptr(), z.data_ptr(), 4,
                                z.data_ptr(), 0, out.data_ptr(), 0))
    assert L.rg_ic_spectrum(None, None, 4, 1, None, None, 4, None, 4, None, 0) == capi.RG_ERR_ARGUMENT


def test_dropin_module(gpu, oracle_lib):
    import ragnar_gb300 as rg  # noqa: PLC0415

    rg.Initialize()
    dist_prtls = rg.TabulatedDistribution(rg.Logbins(1e3, 1e7, 200), rg.PlawGenerator(-1.5, 1e3, 1e7))
    dist_soft = rg.TabulatedDistribution(rg.Logbins(1e-11, 1e-7, 200, rg.EnergyUnits.mec2),
                                         rg.DeltaGenerator(1e-8, 1e-9))
    bins = rg.Bins(rg.Logspace(1e3, 1e7, 200), rg.EnergyUnits.mec2)
    got = rg.ICSpectrum(dist_prtls, dist_soft, bins).as_array()
    g = golden("ic")
    assert max_rel(got, g["case0_ref"]) <= 5e-5
    with pytest.raises(RuntimeError, match="Soft photons energy bins must be in units of mec\\^2"):
        rg.ICSpectrum(dist_prtls, rg.TabulatedDistribution(rg.Logbins(1e-11, 1e-7, 200),
                                                           rg.DeltaGenerator(1e-8, 1e-9)), bins)
    with pytest.raises(RuntimeError, match="E_ic must be in units of mec\\^2"):
        rg.ICSpectrum(dist_prtls, dist_soft, rg.Bins(rg.Logspace(1e3, 1e7, 200)))

"""GPU parity of Particles.energyDistribution through the C ABI: exact integer
counts per bin (the bin index is bit-exact to the reference's double
expression), sums of 1/energy within FP32 rounding of the FP64 oracle, on the
reference fixtures and on edge energies (zero, exactly at bin thresholds,
above the top bin, NaN and infinity), unaligned and ragged sizes.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from helpers import golden, particles

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
capi = pytest.importorskip("ragnar_gb300.capi")


def gpu_hist(ux, uy, uz, bins, log_spaced, fourvel, dev, offset=0):
    bins = np.ascontiguousarray(bins, np.float32)
    n = len(ux)
    T = [torch.from_numpy(np.concatenate([np.zeros(offset, np.float32), a]).astype(np.float32)).to(dev)
         for a in (ux, uy, uz)]
    T = [t[offset:] for t in T]
    hist = torch.full((len(bins),), -1.0, device=dev)
    counts = torch.full((len(bins),), -1, dtype=torch.int64, device=dev)
    capi.check(capi.lib().rg_energy_distribution(T[0].data_ptr(), T[1].data_ptr(), T[2].data_ptr(), n,
                                                 bins.ctypes.data, len(bins), int(log_spaced),
                                                 int(fourvel), hist.data_ptr(), counts.data_ptr(), 0))
    torch.cuda.synchronize()
    return hist.cpu().numpy(), counts.cpu().numpy()


def check_against_oracle(oracle_lib, ux, uy, uz, bins, log_spaced, fourvel, dev, offset=0):
    h, c = gpu_hist(ux, uy, uz, bins, log_spaced, fourvel, dev, offset)
    _, h64, cnt = oracle_lib.energy_distribution(ux, uy, uz, bins, log_spaced, fourvel)
    np.testing.assert_array_equal(c, cnt)
    if log_spaced:
        fin = np.isfinite(h64) & (h64 > 0)
        # FP32 per-block partial sums flushed to FP64: ~1e-7 relative (the
        # reference accumulates in FP32 per thread, ~1e-5)
        assert np.all(np.abs(h[fin] - h64[fin]) <= 1e-6 * h64[fin])
        assert np.array_equal(np.isinf(h), np.isinf(h64))
    else:
        np.testing.assert_array_equal(h, cnt.astype(np.float32))
    return h, c


@pytest.mark.parametrize("case", range(4))
def test_reference_fixtures(gpu, oracle_lib, case):
    g = golden("histogram")
    u = g["u"]
    bins, (logb, fourvel), F = g[f"case{case}_bins"], g[f"case{case}_meta"], g[f"case{case}_F"]
    h, c = check_against_oracle(oracle_lib, u[0], u[1], u[2], bins, bool(logb), bool(fourvel), gpu)
    if logb:
        m = F > 0
        assert np.max(np.abs(h[m] - F[m]) / F[m]) < 1e-5
    else:
        np.testing.assert_array_equal(c, F.astype(np.int64))


@pytest.mark.parametrize("n", [1, 3, 4, 7, 4096, 4099, 100003])
@pytest.mark.parametrize("offset", [0, 1])
def test_sizes_and_alignment(gpu, oracle_lib, n, offset):
    P = particles(n, seed=n + offset)
    bins = oracle_lib.logspace(1e-2, 1e3, 200)
    check_against_oracle(oracle_lib, P["ux"], P["uy"], P["uz"], bins, True, True, gpu, offset)


@pytest.mark.parametrize("log_spaced,fourvel", [(True, True), (True, False), (False, True), (False, False)])
def test_edge_energies(gpu, oracle_lib, log_spaced, fourvel):
    bins = oracle_lib.logspace(0.5, 50.0, 64) if log_spaced else oracle_lib.linspace(0.5, 50.0, 64)
    thr = np.empty(64, np.float32)
    nan_idx = ctypes.c_int32()
    capi.check(capi.lib().rg_energy_thresholds(bins.ctypes.data, 64, int(fourvel), thr.ctypes.data,
                                               ctypes.byref(nan_idx)))
    usq = [0.0, 1e-30, 0.25, 2500.0, 1e6, np.inf]
    for t in thr[1:]:
        if np.isfinite(t):
            usq += [np.nextafter(t, np.float32(0)), t, np.nextafter(t, np.float32(np.inf))]
    usq = np.array(usq, np.float32)
    ux = np.sqrt(usq).astype(np.float32)
    # keep |u|^2 exactly as listed: put it all in one component where sqrt is exact enough
    keep = ux.astype(np.float64) ** 2 == usq.astype(np.float64)
    ux, usq = ux[keep], usq[keep]
    z = np.zeros_like(ux)
    check_against_oracle(oracle_lib, ux, z, z, bins, log_spaced, fourvel, gpu)


@pytest.mark.parametrize("kind", ["log4096", "lin4096", "narrow", "float_overflow"])
@pytest.mark.parametrize("fourvel", [True, False])
def test_bin_lookup_cell_table(gpu, oracle_lib, kind, fourvel):
    """Bin sets whose float-bit cell table holds several thresholds per cell (4096 bins),
    spans a tiny range (1 .. 1.0001), or has no finite threshold at all (bins 1e-30 .. 1e30:
    the reference's float emax / emin overflows, so every finite energy lands in bin 0):
    counts bit-exact against the oracle for random particles and for |u| within 2 ulp of the
    square root of every finite threshold."""
    log_spaced = kind in ("log4096", "float_overflow")
    bins = {"log4096": lambda: oracle_lib.logspace(1e-4, 1e9, 4096),
            "lin4096": lambda: oracle_lib.linspace(0.01, 1e3, 4096),
            "narrow": lambda: oracle_lib.linspace(1.0, 1.0001, 50),
            "float_overflow": lambda: oracle_lib.logspace(1e-30, 1e30, 300)}[kind]()
    nb = len(bins)
    thr = np.empty(nb, np.float32)
    nan_idx = ctypes.c_int32()
    capi.check(capi.lib().rg_energy_thresholds(bins.ctypes.data, nb, int(fourvel), thr.ctypes.data,
                                               ctypes.byref(nan_idx)))
    # |u| within 2 ulp of sqrt(threshold): Usqr = |u|^2 lands on both sides of every threshold
    s = np.sqrt(thr[1:][np.isfinite(thr[1:])].astype(np.float64)).astype(np.float32)
    lo1, hi1 = np.nextafter(s, np.float32(0)), np.nextafter(s, np.float32(np.inf))
    edge = np.concatenate([s, lo1, hi1, np.nextafter(lo1, np.float32(0)), np.nextafter(hi1, np.float32(np.inf)),
                           np.array([0.0, 1e-23, 1e-15, 1.0, 1.7e19, np.inf], np.float32)]).astype(np.float32)
    P = particles(100_000, seed=17)
    z = np.zeros_like(edge)
    ux, uy, uz = (np.concatenate([a, P[k]]) for a, k in ((edge, "ux"), (z, "uy"), (z, "uz")))
    check_against_oracle(oracle_lib, ux, uy, uz, bins, log_spaced, fourvel, gpu)


def test_nan_and_inf_inputs(gpu, oracle_lib):
    ux = np.array([np.nan, np.inf, -np.inf, 3.0, 0.0], np.float32)
    z = np.zeros_like(ux)
    bins = oracle_lib.logspace(1e-2, 1e3, 50)
    h, c = gpu_hist(ux, z, z, bins, False, True, gpu)
    _, _, cnt = oracle_lib.energy_distribution(ux, z, z, bins, False, True)
    np.testing.assert_array_equal(c, cnt)
    assert c.sum() == len(ux)


def test_full_size_counts_conserved(gpu):
    """1e8 particles: every particle lands in exactly one bin, and two halves add up."""
    n = 100_000_000
    gen = torch.Generator(device=gpu).manual_seed(1)
    u = [torch.randn(n, device=gpu, generator=gen) * 30 for _ in range(3)]
    bins = np.logspace(-2, 3, 200).astype(np.float32)

    def run(lo, hi):
        hist = torch.empty(200, device=gpu)
        counts = torch.empty(200, dtype=torch.int64, device=gpu)
        capi.check(capi.lib().rg_energy_distribution(u[0][lo:].data_ptr(), u[1][lo:].data_ptr(),
                                                     u[2][lo:].data_ptr(), hi - lo, bins.ctypes.data, 200,
                                                     1, 1, hist.data_ptr(), counts.data_ptr(), 0))
        torch.cuda.synchronize()
        return hist.double().cpu().numpy(), counts.cpu().numpy()

    h, c = run(0, n)
    h1, c1 = run(0, 40_000_000)
    h2, c2 = run(40_000_000, n)
    assert c.sum() == n
    np.testing.assert_array_equal(c, c1 + c2)
    m = h > 0
    assert np.max(np.abs(h1[m] + h2[m] - h[m]) / h[m]) < 1e-6


def test_threshold_cache_eviction(gpu, oracle_lib):
    """More bin sets than the device threshold cache keeps (16): evicted sets are rebuilt
    and every call still matches the oracle bit for bit."""
    P = particles(20000, seed=33)
    for rep in range(2):
        for i in range(20):
            bins = oracle_lib.logspace(1e-2 * (1.0 + 0.01 * i), 1e3, 50 + i)
            h, c = gpu_hist(P["ux"], P["uy"], P["uz"], bins, True, True, gpu)
            _, h64, cnt = oracle_lib.energy_distribution(P["ux"], P["uy"], P["uz"], bins, True, True)
            np.testing.assert_array_equal(c, cnt)


def test_more_than_2_pow_31_particles(gpu):
    """2^31 + 12345 particles (26 GB of u): 64-bit indexing; every particle is counted once
    and two halves add up to the whole."""
    n = (1 << 31) + 12345
    gen = torch.Generator(device=gpu).manual_seed(11)
    u = [torch.rand(n, device=gpu, generator=gen) * 20 - 10 for _ in range(3)]
    bins = np.logspace(-2, 3, 100).astype(np.float32)

    def run(lo, hi):
        hist = torch.empty(100, device=gpu)
        counts = torch.empty(100, dtype=torch.int64, device=gpu)
        capi.check(capi.lib().rg_energy_distribution(u[0][lo:].data_ptr(), u[1][lo:].data_ptr(),
                                                     u[2][lo:].data_ptr(), hi - lo, bins.ctypes.data, 100,
                                                     1, 1, hist.data_ptr(), counts.data_ptr(), 0))
        torch.cuda.synchronize()
        return hist.double().cpu().numpy(), counts.cpu().numpy()

    h, c = run(0, n)
    h1, c1 = run(0, 1 << 30)
    h2, c2 = run(1 << 30, n)
    del u
    torch.cuda.empty_cache()
    assert int(c.sum()) == n
    np.testing.assert_array_equal(c, c1 + c2)
    m = h > 0
    assert np.max(np.abs(h1[m] + h2[m] - h[m]) / h[m]) < 1e-6

"""The interval-moment spectrum (moments.cu) against the fused kernel and the oracle.

Both sum the reference's sync::Kernel (synchrotron.hpp:145-172) over particles
and bins with the same fixed-point table coordinate; interval moments sum the
piecewise-linear F exactly in FP64 per (table cell, bin interval) instead of
evaluating every (particle, bin) pair in FP32.  Checked here: which plans and
runs take the path, agreement with the fused kernel and the FP64 oracle on
bin sets whose low parts tie or crowd one bucket, 256 uneven segments with
empty ones, and the fallback above 1024 segments.
"""

from __future__ import annotations

import numpy as np
import pytest

from helpers import SPECTRUM_RTOL, max_rel, particles

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
capi = pytest.importorskip("ragnar_gb300.capi")


def _device(P, dev):
    T = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in P.items()}
    prt = capi.particles([T["ux"], T["uy"], T["uz"]], b=[T["bx"], T["by"], T["bz"]],
                         e=[T["ex"], T["ey"], T["ez"]] if "ex" in T else None, w=T.get("w"), n=len(P["ux"]))
    return T, prt


@pytest.fixture(scope="module")
def table(oracle_lib):
    return oracle_lib.tabulate_ffunc()


def test_algorithm_selection(gpu, oracle_lib):
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    ref = capi.SpectrumPlan(bins, 1.0, 1.0, 1.0)
    assert ref.algorithm(1) == capi.RG_ALGO_MOMENTS
    assert ref.algorithm(1024) == capi.RG_ALGO_MOMENTS
    assert ref.algorithm(1025) == capi.RG_ALGO_DIRECT  # more segments than the deposit stages
    ref.set_algorithm(capi.RG_ALGO_DIRECT)
    assert ref.algorithm(1) == capi.RG_ALGO_DIRECT
    with pytest.raises(capi.RgError):
        ref.set_algorithm(7)
    # smooth table: moments over log-uniform bins (the plan's bin-aligned table) only
    assert capi.SpectrumPlan(bins, 1.0, 1.0, 1.0, capi.RG_TABLE_SMOOTH).algorithm(1) == capi.RG_ALGO_MOMENTS
    uneven = np.sort(np.concatenate([bins[:100], bins[100:] * 1.01])).astype(np.float32)
    smooth = capi.SpectrumPlan(uneven, 1.0, 1.0, 1.0, capi.RG_TABLE_SMOOTH)
    assert smooth.algorithm(1) == capi.RG_ALGO_DIRECT
    smooth.set_algorithm(capi.RG_ALGO_MOMENTS)
    P = particles(100, seed=1)
    T, prt = _device(P, gpu)
    out = torch.empty(200, device=gpu)
    with pytest.raises(capi.RgError) as e:
        smooth.run(prt, out)
    assert e.value.status == capi.RG_ERR_UNSUPPORTED


@pytest.mark.parametrize("kind", ["log512", "ties", "one_bucket", "linear", "sparse"])
def test_moments_vs_fused_and_oracle(gpu, oracle_lib, table, kind):
    P = particles(40000, seed=["log512", "ties", "one_bucket", "linear", "sparse"].index(kind) + 70, bfield="iso", weights=True, efield=kind == "linear",
                  umax=1e4, index=-2.2)
    if kind == "log512":
        bins = oracle_lib.logspace(1e-4, 1e9, 512)
    elif kind == "ties":  # repeated bins: equal low parts
        bins = np.repeat(oracle_lib.logspace(1e-2, 1e6, 50), 4).astype(np.float32)
    elif kind == "one_bucket":  # bins a whole number of table segments apart: low parts crowd one bucket
        xs, _ = table
        r = float(xs[1]) / float(xs[0])
        bins = (0.5 * r ** np.arange(0, 300, 3)).astype(np.float32)
    elif kind == "linear":
        bins = oracle_lib.linspace(-10.0, 5000.0, 333)
    else:  # few bins far apart, some outside every particle's reach
        bins = np.array([1e-12, 1e-3, 7.0, 3e4, 2e9, 1e15], np.float32)
    T, prt = _device(P, gpu)
    res = {}
    for algo in (capi.RG_ALGO_DIRECT, capi.RG_ALGO_MOMENTS):
        plan = capi.SpectrumPlan(bins, 1.0, 1.0, 1.0)
        plan.set_algorithm(algo)
        out = torch.full((len(bins),), -1.0, device=gpu)
        plan.run(prt, out)
        plan.check()
        res[algo] = out.cpu().numpy()
        plan.close()
    truth = oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table)
    got = res[capi.RG_ALGO_MOMENTS]
    assert max_rel(got, truth) <= SPECTRUM_RTOL
    assert np.array_equal(got == 0, truth == 0)
    assert max_rel(got, res[capi.RG_ALGO_DIRECT]) <= SPECTRUM_RTOL


def test_moments_256_uneven_segments(gpu, oracle_lib, table):
    rng = np.random.default_rng(256)
    counts = np.floor(10.0 ** rng.uniform(0.0, 3.5, 256)).astype(np.int64)
    counts[[3, 100, 101, 255]] = 0
    offs = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    n = int(offs[-1])
    P = particles(n, seed=257, bfield="iso", weights=True)
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    T, prt = _device(P, gpu)
    plan = capi.SpectrumPlan(bins, 1.0, 1.0, 1.0)
    plan.reserve(256)
    assert plan.algorithm(256) == capi.RG_ALGO_MOMENTS
    out = torch.empty((256, 200), device=gpu)
    plan.run_batched(prt, torch.from_numpy(offs).to(gpu), 256, out)
    plan.check()
    got = out.cpu().numpy()
    truth = oracle_lib.sync_spectrum_batched_f64(P, offs, bins, 1.0, 1.0, 1.0, table)
    for s in range(256):
        if counts[s] == 0:
            assert np.all(got[s] == 0)
        else:
            assert max_rel(got[s], truth[s]) <= SPECTRUM_RTOL, s


def test_more_segments_than_staged_fall_back_to_fused(gpu, oracle_lib, table):
    nseg = 1100
    offs = np.arange(0, 5 * nseg + 1, 5, dtype=np.int64)
    P = particles(int(offs[-1]), seed=1100, bfield="iso")
    bins = oracle_lib.logspace(0.01, 1e7, 64)
    T, prt = _device(P, gpu)
    plan = capi.SpectrumPlan(bins, 1.0, 1.0, 1.0)
    plan.reserve(nseg)
    assert plan.algorithm(nseg) == capi.RG_ALGO_DIRECT
    out = torch.empty((nseg, 64), device=gpu)
    plan.run_batched(prt, torch.from_numpy(offs).to(gpu), nseg, out)
    plan.check()
    truth = oracle_lib.sync_spectrum_batched_f64(P, offs, bins, 1.0, 1.0, 1.0, table)
    got = out.cpu().numpy()
    for s in (0, 1, 517, nseg - 1):
        assert max_rel(got[s], truth[s]) <= SPECTRUM_RTOL


@pytest.mark.parametrize("B0,eps,negw", [(1.0, 1.0, True), (-2.0, -1.5, False)])
def test_negative_amplitudes(gpu, oracle_lib, table, B0, eps, negw):
    """Negative weights, or B0 and e_syn_at_g_syn both negative (K0 > 0, amplitude
    1/B0 < 0): every particle still adds its (signed) term, as in the reference's sum."""
    P = particles(30000, seed=88, bfield="iso", weights=True)
    if negw:
        P["w"][::3] *= -1.0
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    T, prt = _device(P, gpu)
    res = {}
    for algo in (capi.RG_ALGO_DIRECT, capi.RG_ALGO_MOMENTS):
        plan = capi.SpectrumPlan(bins, B0, 1.0, eps)
        plan.set_algorithm(algo)
        out = torch.empty(200, device=gpu)
        plan.run(prt, out)
        plan.check()
        res[algo] = out.cpu().numpy().astype(np.float64)
    truth = oracle_lib.sync_spectrum_f64(P, bins, B0, 1.0, eps, table)
    scale = np.abs(truth).max()
    for algo, got in res.items():
        # signed sums can cancel: compare against the largest magnitude
        assert np.max(np.abs(got - truth)) <= SPECTRUM_RTOL * scale, algo

"""Many distributions at once on the tensor cores (rg_fromdist_*): the BF16
split-precision tcgen05 GEMM against the FP64 oracle of SynchrotronSpectrumFromDist
(synchrotron.cpp:69-105, synchrotron.hpp:72-95), its transpose GEMM (the adjoint)
against K^T in FP64, the torch.autograd binding, ragged shapes across the
128 x 256 tile edges and argument checks."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import SPECTRUM_RTOL, max_rel

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
capi = pytest.importorskip("ragnar_gb300.capi")
rt = pytest.importorskip("ragnar_gb300.torch_ext")


def _dists(gb, ndist, seed):
    """Power laws with random index and exponential cutoff, one per row."""
    rng = np.random.default_rng(seed)
    g = gb.astype(np.float64)[None, :]
    p = rng.uniform(1.5, 3.5, (ndist, 1))
    gc = 10.0 ** rng.uniform(1.0, 4.5, (ndist, 1))
    amp = 10.0 ** rng.uniform(-2.0, 2.0, (ndist, 1))
    return (amp * g**-p * np.exp(-g / gc)).astype(np.float32)


def _run(plan, f, dev):
    ft = torch.from_numpy(f).to(dev)
    out = torch.empty((f.shape[0], plan.nbins), device=dev)
    plan.run(ft, out)
    plan.check()
    return out.cpu().numpy()


def _rows_max_rel(S, S64):
    return max(max_rel(S[d], S64[d]) for d in range(S.shape[0]))


@pytest.fixture(scope="module")
def table(oracle_lib):
    return oracle_lib.tabulate_ffunc()


@pytest.mark.parametrize("log_spaced", [True, False])
def test_gemm_matches_fp64_oracle(gpu, oracle_lib, table, log_spaced):
    gb = oracle_lib.logspace(1.0, 1e5, 300) if log_spaced else oracle_lib.linspace(1.0, 3e3, 300)
    bins = oracle_lib.logspace(0.01, 1e11, 400)
    f = _dists(gb, 200, seed=3 + log_spaced)
    plan = capi.FromDistPlan(gb, log_spaced, bins, 1.0, 1.0, max_dist=256)
    S = _run(plan, f, gpu)
    S64 = oracle_lib.sync_from_dist_f64(gb, f, log_spaced, bins, 1.0, 1.0, table)
    assert _rows_max_rel(S, S64) <= SPECTRUM_RTOL
    # the FP64 kernel matrix the plan built, against the oracle's one-hot spectra
    K = plan.kernel_matrix()
    eye = np.zeros((3, len(gb)), np.float32)
    for i, g in enumerate((0, 150, 299)):
        eye[i, g] = 1.0
    K64 = oracle_lib.sync_from_dist_f64(gb, eye, log_spaced, bins, 1.0, 1.0, table)
    for i, g in enumerate((0, 150, 299)):
        assert max_rel(bins.astype(np.float64) * K[:, g], K64[i]) <= SPECTRUM_RTOL


def test_three_products_fast_mode(gpu, oracle_lib, table):
    gb = oracle_lib.logspace(1.0, 1e5, 256)
    bins = oracle_lib.logspace(0.01, 1e11, 256)
    f = _dists(gb, 64, seed=11)
    S64 = oracle_lib.sync_from_dist_f64(gb, f, True, bins, 1.0, 1.0, table)
    plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=64, split_products=3)
    # two BF16 terms per operand keep ~16 significant bits of each product
    assert _rows_max_rel(_run(plan, f, gpu), S64) <= 1e-4


@pytest.mark.parametrize("ndist,ng,nbins", [(1, 77, 1), (129, 64, 257), (300, 513, 600), (5, 2, 33)])
def test_ragged_shapes(gpu, oracle_lib, table, ndist, ng, nbins):
    gb = oracle_lib.logspace(1.0, 1e4, ng)
    bins = oracle_lib.logspace(0.1, 1e9, nbins) if nbins > 1 else np.array([100.0], np.float32)
    f = _dists(gb, ndist, seed=ndist + ng)
    plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=ndist)
    S = _run(plan, f, gpu)
    S64 = oracle_lib.sync_from_dist_f64(gb, f, True, bins, 1.0, 1.0, table)
    assert S.shape == (ndist, nbins)
    assert _rows_max_rel(S, S64) <= SPECTRUM_RTOL


def test_fewer_distributions_than_planned_and_invalid_bins(gpu, oracle_lib, table):
    gb = oracle_lib.logspace(1.0, 1e5, 200)
    bins = oracle_lib.logspace(0.01, 1e11, 300)
    bins[[0, 7, 299]] = [0.0, -1.0, np.nan]  # non-positive / NaN photon energies give 0
    f = _dists(gb, 40, seed=5)
    plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=1000)
    S = _run(plan, f, gpu)
    good = np.ones(300, bool)
    good[[0, 7, 299]] = False
    assert np.all(S[:, ~good] == 0.0)
    S64 = oracle_lib.sync_from_dist_f64(gb, f, True, bins[good], 1.0, 1.0, table)
    assert _rows_max_rel(S[:, good], S64) <= SPECTRUM_RTOL


def test_adjoint_is_transpose(gpu, oracle_lib):
    gb = oracle_lib.logspace(1.0, 1e5, 300)
    bins = oracle_lib.logspace(0.01, 1e11, 400)
    plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=128, mode=capi.RG_TABLE_SMOOTH)
    K = plan.kernel_matrix()  # FP64 [nbins, ng]
    rng = np.random.default_rng(9)
    gS = rng.standard_normal((100, 400)).astype(np.float32)
    gf = torch.empty((100, 300), device=gpu)
    plan.adjoint(torch.from_numpy(gS).to(gpu), gf)
    plan.check()
    want = (gS.astype(np.float64) * bins.astype(np.float64)[None, :]) @ K
    got = gf.cpu().numpy()
    scale = np.max(np.abs(want), axis=1, keepdims=True)
    assert np.max(np.abs(got - want) / scale) < 1e-5


def test_smooth_mode_matches_single_distribution_path(gpu, oracle_lib):
    gb = oracle_lib.logspace(1.0, 1e5, 300)
    bins = oracle_lib.logspace(0.01, 1e11, 400)
    f = _dists(gb, 16, seed=17)
    plan = rt.fromdist_plan(gb, bins, max_dist=16)
    S = rt.synchrotron_from_dist_batched(plan, torch.from_numpy(f).to(gpu)).cpu().numpy()
    one = rt.dist_plan(bins)
    g_t = torch.from_numpy(gb).to(gpu)
    for d in (0, 5, 15):
        ref = rt.synchrotron_from_dist(one, g_t, torch.from_numpy(f[d]).to(gpu)).cpu().numpy()
        assert max_rel(S[d], ref) <= 2 * SPECTRUM_RTOL


def test_autograd(gpu, oracle_lib):
    gb = oracle_lib.logspace(1.0, 1e5, 200)
    bins = oracle_lib.logspace(0.01, 1e11, 256)
    plan = rt.fromdist_plan(gb, bins, max_dist=32)
    f = torch.from_numpy(_dists(gb, 32, seed=23)).to(gpu).requires_grad_(True)
    w = torch.rand((32, 256), device=gpu)
    (rt.synchrotron_from_dist_batched(plan, f) * w).sum().backward()
    K = plan.kernel_matrix()
    want = (w.cpu().numpy().astype(np.float64) * bins.astype(np.float64)[None, :]) @ K
    got = f.grad.cpu().numpy()
    assert np.max(np.abs(got - want) / np.max(np.abs(want), axis=1, keepdims=True)) < 1e-5


def test_arguments(gpu, oracle_lib):
    gb = oracle_lib.logspace(1.0, 1e3, 10)
    bins = oracle_lib.logspace(0.1, 1e3, 10)
    with pytest.raises(capi.RgError, match="split_products"):
        capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=4, split_products=4)
    plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=4)
    f = torch.ones((5, 10), device=gpu)
    out = torch.empty((5, 10), device=gpu)
    with pytest.raises(capi.RgError, match="max_dist"):
        plan.run(f, out)
    plan.run(f[:0], out[:0])  # no distributions: nothing to do
    plan.check()


def test_long_k_accumulation_stays_within_tolerance(gpu, oracle_lib):
    """1024 gamma bins (6 x 1024 concatenated K, 384 MMA steps) on 1024 photon bins over
    15 decades: the FP32 accumulation must still meet the spectrum tolerance."""
    gb = oracle_lib.logspace(1.0, 1e6, 1024)
    bins = oracle_lib.logspace(1e-2, 1e13, 1024)
    rng = np.random.default_rng(505)
    g = gb.astype(np.float64)[None, :]
    p = rng.uniform(-3.0, -1.5, (256, 1))
    lo = 10.0 ** rng.uniform(0.0, 2.0, (256, 1))
    hi = 10.0 ** rng.uniform(3.0, 6.0, (256, 1))
    f = np.where((g >= lo) & (g < hi), g**p, 0.0).astype(np.float32)
    plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=256)
    S = _run(plan, f, gpu).astype(np.float64)
    S64 = (f.astype(np.float64) @ plan.kernel_matrix().T) * bins.astype(np.float64)[None, :]
    assert _rows_max_rel(S, S64) <= SPECTRUM_RTOL


@pytest.mark.parametrize("cfg", [0, 1, 2])
def test_every_tile_shape(gpu, oracle_lib, table, cfg):
    """Each shape the autotuner may pick, forced, on sizes with partial tiles in M and N."""
    gb = oracle_lib.logspace(1.0, 1e4, 300)
    bins = oracle_lib.logspace(0.1, 1e9, 300)
    f = _dists(gb, 200, seed=40 + cfg)
    plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=200)
    tuned = plan.config()
    shapes = [(256, 4), (128, 6), (128, 4)]
    assert tuned["fwd"] in shapes and tuned["adj"] in shapes
    plan.set_config(cfg, cfg)
    S = _run(plan, f, gpu)
    S64 = oracle_lib.sync_from_dist_f64(gb, f, True, bins, 1.0, 1.0, table)
    assert _rows_max_rel(S, S64) <= SPECTRUM_RTOL
    gS = np.random.default_rng(cfg).standard_normal((200, 300)).astype(np.float32)
    gf = torch.empty((200, 300), device=gpu)
    plan.adjoint(torch.from_numpy(gS).to(gpu), gf)
    plan.check()
    want = (gS.astype(np.float64) * bins.astype(np.float64)[None, :]) @ plan.kernel_matrix()
    assert np.max(np.abs(gf.cpu().numpy() - want) / np.max(np.abs(want), axis=1, keepdims=True)) < 1e-5
    with pytest.raises(capi.RgError, match="out of range"):
        plan.set_config(3, 0)


@pytest.mark.parametrize("split", [1, 2, 4, 8])
@pytest.mark.parametrize("ng,nbins", [(600, 520), (601, 522)])
def test_every_split_k(gpu, oracle_lib, table, split, ng, nbins):
    """Split-K forced to each count the autotuner may pick: the ranges' products summed in
    range order match the FP64 oracle (forward) and K^T (adjoint), and reruns are
    bit-identical; row lengths that are multiples of 4 take the tensor-store epilogue, the
    others the direct stores."""
    gb = oracle_lib.logspace(1.0, 1e5, ng)   # 10 k blocks of 64
    bins = oracle_lib.logspace(0.01, 1e11, nbins)  # 9 k blocks for the adjoint
    f = _dists(gb, 130, seed=70 + split)
    plan = capi.FromDistPlan(gb, True, bins, 1.0, 1.0, max_dist=130)
    assert plan.split_k()["fwd"] in (1, 2, 4, 8) and plan.split_k()["adj"] in (1, 2, 4, 8)
    plan.set_split_k(split, split)
    assert plan.split_k() == {"fwd": split, "adj": split}
    S = _run(plan, f, gpu)
    S64 = oracle_lib.sync_from_dist_f64(gb, f, True, bins, 1.0, 1.0, table)
    assert _rows_max_rel(S, S64) <= SPECTRUM_RTOL
    assert np.array_equal(S, _run(plan, f, gpu))
    gS = np.random.default_rng(split).standard_normal((130, nbins)).astype(np.float32)
    gf = torch.empty((130, ng), device=gpu)
    plan.adjoint(torch.from_numpy(gS).to(gpu), gf)
    plan.check()
    want = (gS.astype(np.float64) * bins.astype(np.float64)[None, :]) @ plan.kernel_matrix()
    assert np.max(np.abs(gf.cpu().numpy() - want) / np.max(np.abs(want), axis=1, keepdims=True)) < 1e-5
    for bad in ((3, -1), (16, -1), (-1, 16)):
        with pytest.raises(capi.RgError, match="counts are 1, 2, 4 or 8"):
            plan.set_split_k(*bad)


def test_forward_and_adjoint_replay_from_cuda_graph(gpu, oracle_lib):
    """The split + GEMM forward and the transpose-GEMM adjoint make no host
    synchronisation or allocation, so a training step can be captured once and replayed."""
    gb = oracle_lib.logspace(1.0, 1e5, 200)
    bins = oracle_lib.logspace(0.01, 1e11, 256)
    plan = rt.fromdist_plan(gb, bins, max_dist=64)
    f = torch.from_numpy(_dists(gb, 64, seed=31)).to(gpu)
    w = torch.rand((64, 256), device=gpu)
    S = torch.empty((64, 256), device=gpu)
    gf = torch.empty((64, 200), device=gpu)
    stream = torch.cuda.current_stream(gpu).cuda_stream
    plan.run(f, S, stream)  # warm (configures the kernels) outside the capture
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        s = torch.cuda.current_stream(gpu).cuda_stream
        plan.run(f, S, s)
        plan.adjoint(w, gf, s)
    f.mul_(2.0)  # replays read the inputs as they are at replay time
    graph.replay()
    plan.check()
    S_ref = torch.empty_like(S)
    gf_ref = torch.empty_like(gf)
    plan.run(f, S_ref)
    plan.adjoint(w, gf_ref)
    plan.check()
    assert torch.equal(S, S_ref) and torch.equal(gf, gf_ref)

"""GPU parity of the particle spectrum, called through the C ABI.

Both ways of summing the spectrum -- the fused kernel (RG_ALGO_DIRECT, every
(particle, bin) pair in FP32) and interval moments (RG_ALGO_MOMENTS, the default
for reference-table particle plans) -- are compared with the oracle's FP64
ground truth (1e-5 relative on bins above 1e-12 of the peak) and with the
reference's own outputs (golden fixtures), on the reference's edge cases: empty
and tiny inputs, sizes around the chunk and warp boundaries, bins that are not
log-spaced or not positive, particles with no emission (u = 0, u parallel to
B), E fields, weights, unaligned streams; plus the batched launch and
size-independent properties at full size (additivity over segments, exact
power-of-two scaling, reruns: bit-identical for the fused kernel, equal to FP64
rounding for interval moments, whose FP64 atomic sums do not fix the order).
"""

from __future__ import annotations

import numpy as np
import pytest

from helpers import SPECTRUM_RTOL, golden, max_rel, particles

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
capi = pytest.importorskip("ragnar_gb300.capi")


def to_device(P, dev):
    T = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in P.items()}
    prt = capi.particles([T["ux"], T["uy"], T["uz"]],
                         b=[T.get("bx"), T.get("by"), T.get("bz")],
                         e=[T.get("ex"), T.get("ey"), T.get("ez")] if "ex" in T else None,
                         w=T.get("w"), n=len(P["ux"]))
    return T, prt


ALGOS = [pytest.param(1, id="direct"), pytest.param(2, id="moments")]


@pytest.fixture(params=ALGOS)
def algo(request):
    return request.param


def make_plan(bins, B0=1.0, g=1.0, eps=1.0, algo=0):
    plan = capi.SpectrumPlan(bins, B0, g, eps)
    plan.set_algorithm(algo)
    return plan


def same(a, b, algo):
    """Reruns: bit-identical for the fused kernel; for interval moments equal up to the
    FP64 rounding of the atomic sums (so in FP32 to within one rounding)."""
    if algo == capi.RG_ALGO_DIRECT:
        assert torch.equal(a, b)
    else:
        a64, b64 = a.double(), b.double()
        scale = torch.clamp(b64.abs(), min=1e-300)
        assert bool(((a64 - b64).abs() <= 1.2e-7 * scale).all())


def gpu_spectrum(P, bins, dev, B0=1.0, g=1.0, eps=1.0, plain=False, algo=0):
    T, prt = to_device(P, dev)
    plan = make_plan(bins, B0, g, eps, algo)
    out = torch.full((len(bins),), -1.0, device=dev)
    (plan.run_plain if plain else plan.run)(prt, out)
    plan.check()
    res = out.cpu().numpy()
    plan.close()
    return res


@pytest.fixture(scope="module")
def table(oracle_lib):
    return oracle_lib.tabulate_ffunc()


@pytest.mark.parametrize("case", ["c1", "iso", "efield"])
def test_matches_reference_fixtures(gpu, oracle_lib, table, case, algo):
    g = golden("spectrum")
    u, b, e = g[f"{case}_u"], g[f"{case}_b"], g[f"{case}_e"]
    P = {"ux": u[0], "uy": u[1], "uz": u[2], "bx": b[0], "by": b[1], "bz": b[2]}
    if np.any(e != 0):
        P.update(ex=e[0], ey=e[1], ez=e[2])
    bins, ref = g[f"{case}_bins"], g[f"{case}_ref"]
    got = gpu_spectrum(P, bins, gpu, algo=algo)
    truth = oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table)
    assert max_rel(got, truth) <= SPECTRUM_RTOL
    # vs the reference itself: GPU error plus the reference's own FP32 error
    assert max_rel(got, ref) <= SPECTRUM_RTOL + max_rel(ref, truth)
    assert np.array_equal(got == 0, ref == 0)


@pytest.mark.parametrize("n", [0, 1, 3, 4, 5, 511, 512, 513, 1025, 4099])
@pytest.mark.parametrize("nbins", [1, 31, 32, 33, 200])
def test_sizes_and_edges(gpu, oracle_lib, table, n, nbins, algo):
    P = particles(max(n, 1), seed=n * 7 + nbins, bfield="iso")
    if n == 0:
        P = {k: v[:0] for k, v in P.items()}
    bins = oracle_lib.logspace(0.01, 1e7, nbins) if nbins > 1 else np.array([3.0], np.float32)
    got = gpu_spectrum(P, bins, gpu, algo=algo)
    truth = oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table) if n else np.zeros(nbins)
    assert got.shape == (nbins,)
    assert max_rel(got, truth) <= SPECTRUM_RTOL
    assert np.all(got[truth == 0] == 0)


@pytest.mark.parametrize("nbins,lo,hi", [(512, 1e-4, 1e9), (513, 1e-4, 1e9), (1024, 1e-2, 1e13),
                                          (1500, 1e-3, 1e8)])
def test_many_bins_and_slices(gpu, oracle_lib, table, nbins, lo, hi, algo):
    P = particles(20000, seed=nbins, bfield="iso", weights=True, umax=1e4, index=-2.2)
    bins = oracle_lib.logspace(lo, hi, nbins)
    got = gpu_spectrum(P, bins, gpu, algo=algo)
    assert max_rel(got, oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table)) <= SPECTRUM_RTOL


def test_linear_and_nonpositive_bins(gpu, oracle_lib, table, algo):
    P = particles(5000, seed=3, bfield="iso")
    bins = oracle_lib.linspace(-5.0, 300.0, 250)  # includes negative and zero-crossing bins
    got = gpu_spectrum(P, bins, gpu, algo=algo)
    truth = oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table)
    assert np.all(got[bins <= 0] == 0)
    assert max_rel(got, truth) <= SPECTRUM_RTOL


def test_non_emitting_particles(gpu, oracle_lib, table, algo):
    n = 3000
    P = particles(n, seed=5)
    P["ux"][:1000] = 0.0  # at rest: chiR = 0 without E
    P["uy"][:1000] = 0.0
    P["uz"][:1000] = 0.0
    P["ux"][1000:2000] = 0.0  # moving along B: u x B = 0
    P["uy"][1000:2000] = 0.0
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    got = gpu_spectrum(P, bins, gpu, algo=algo)
    truth = oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table)
    only = oracle_lib.sync_spectrum_f64({k: v[2000:] for k, v in P.items()}, bins, 1.0, 1.0, 1.0, table)
    np.testing.assert_allclose(truth, only, rtol=1e-12)
    assert max_rel(got, truth) <= SPECTRUM_RTOL


@pytest.mark.parametrize("B0,g,eps", [(0.5, 2.0, 3.0), (3.0, 0.7, 137 * 27 / 8 * 0.1), (1.0, 1.0, -1.0)])
def test_scalars(gpu, oracle_lib, table, B0, g, eps, algo):
    P = particles(4000, seed=11, bfield="iso", efield=True, weights=True)
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    got = gpu_spectrum(P, bins, gpu, B0, g, eps, algo=algo)
    truth = oracle_lib.sync_spectrum_f64(P, bins, B0, g, eps, table)
    if eps < 0:  # e_peak < 0 for every particle: the reference adds nothing
        assert np.all(got == 0) and np.all(truth == 0)
    else:
        assert max_rel(got, truth) <= SPECTRUM_RTOL


def test_unaligned_streams_take_plain_loads(gpu, oracle_lib, table, algo):
    P = particles(10001, seed=2, bfield="iso", weights=True)
    T = {k: torch.from_numpy(np.concatenate([[0.0], v]).astype(np.float32)).to(gpu) for k, v in P.items()}
    # views starting one float in: 4-byte aligned, not 16-byte aligned
    prt = capi.particles([T["ux"][1:], T["uy"][1:], T["uz"][1:]], b=[T["bx"][1:], T["by"][1:], T["bz"][1:]],
                         w=T["w"][1:], n=10001)
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    plan = make_plan(bins, algo=algo)
    out = torch.empty(200, device=gpu)
    plan.run(prt, out)
    plan.check()
    assert max_rel(out.cpu().numpy(), oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table)) <= SPECTRUM_RTOL


def test_plain_kernel(gpu, oracle_lib, table):
    P = particles(30000, seed=4, bfield="iso", weights=True)
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    got = gpu_spectrum(P, bins, gpu, plain=True)
    # FP32 kinematics and log10f interpolation per eval, as the reference writes them
    assert max_rel(got, oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table)) < 2e-4


def test_batched_segments(gpu, oracle_lib, table, algo):
    P = particles(60000, seed=8, bfield="iso", weights=True)
    offs = np.array([0, 0, 1, 100, 100, 513, 5000, 20000, 20003, 60000], np.int64)
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    T, prt = to_device(P, gpu)
    plan = make_plan(bins, algo=algo)
    nseg = len(offs) - 1
    plan.reserve(nseg)
    out = torch.empty((nseg, 200), device=gpu)
    plan.run_batched(prt, torch.from_numpy(offs).to(gpu), nseg, out)
    plan.check()
    got = out.cpu().numpy()
    truth = oracle_lib.sync_spectrum_batched_f64(P, offs, bins, 1.0, 1.0, 1.0, table)
    for s in range(nseg):
        if offs[s + 1] == offs[s]:
            assert np.all(got[s] == 0)
        else:
            assert max_rel(got[s], truth[s]) <= SPECTRUM_RTOL, s


def test_batched_run_replays_from_cuda_graph(gpu, oracle_lib, table, algo):
    """The batched launch captured once into a CUDA graph: each replay reads the
    particle streams and offsets as they are at replay time."""
    P = particles(50000, seed=12, bfield="iso", weights=True)
    bins = oracle_lib.logspace(0.01, 1e7, 300)
    T, prt = to_device(P, gpu)
    plan = make_plan(bins, algo=algo)
    plan.reserve(4)
    offs = torch.tensor([0, 7000, 7000, 31000, 50000], dtype=torch.int64, device=gpu)
    out = torch.empty((4, 300), device=gpu)
    side = torch.cuda.Stream(gpu)
    side.wait_stream(torch.cuda.current_stream(gpu))
    with torch.cuda.stream(side):
        plan.run_batched(prt, offs, 4, out, side.cuda_stream)
    torch.cuda.current_stream(gpu).wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        plan.run_batched(prt, offs, 4, out, torch.cuda.current_stream(gpu).cuda_stream)
    for scale, cuts in ((1.0, [0, 7000, 7000, 31000, 50000]), (0.5, [0, 100, 25000, 25001, 50000])):
        T["w"].copy_(torch.from_numpy(P["w"] * np.float32(scale)))
        offs.copy_(torch.tensor(cuts, dtype=torch.int64))
        graph.replay()
        plan.check()
        eager = torch.empty_like(out)
        plan.run_batched(prt, offs, 4, eager)
        plan.check()
        same(out, eager, algo)
        Pw = dict(P, w=P["w"] * np.float32(scale))
        truth = oracle_lib.sync_spectrum_batched_f64(Pw, np.array(cuts, np.int64), bins, 1.0, 1.0, 1.0, table)
        got = out.cpu().numpy()
        for s in range(4):
            if cuts[s + 1] == cuts[s]:
                assert np.all(got[s] == 0)
            else:
                assert max_rel(got[s], truth[s]) <= SPECTRUM_RTOL, (scale, s)


def test_batched_rejects_bad_offsets(gpu, oracle_lib, algo):
    P = particles(1000, seed=1)
    T, prt = to_device(P, gpu)
    plan = make_plan(oracle_lib.logspace(0.01, 1e7, 64), algo=algo)
    plan.reserve(3)
    out = torch.empty((3, 64), device=gpu)
    for offs in ([0, 500, 400, 1000], [0, 10, 20, 1001]):
        plan.run_batched(prt, torch.tensor(offs, dtype=torch.int64, device=gpu), 3, out)
        with pytest.raises(capi.RgError, match="offsets"):
            plan.check()
    # the plan is usable again after the failure was reported
    plan.run_batched(prt, torch.tensor([0, 10, 20, 1000], dtype=torch.int64, device=gpu), 3, out)
    plan.check()
    assert torch.isfinite(out).all()


def test_stage_wait_timeout_is_reported_and_recoverable(gpu, oracle_lib):
    """A bounded wait that gives up (a barrier phase nothing completes) surfaces as
    RG_ERR_TIMEOUT at the next check; the record clears and the context keeps working."""
    P = particles(2000, seed=4)
    T, prt = to_device(P, gpu)
    plan = make_plan(oracle_lib.logspace(0.01, 1e7, 64), algo=capi.RG_ALGO_DIRECT)
    ref = torch.empty(64, device=gpu)
    plan.run(prt, ref)
    plan.check()
    with pytest.raises(capi.RgError, match="out of range|polls"):
        plan.probe_stage_timeout(0)
    plan.probe_stage_timeout(256)
    with pytest.raises(capi.RgError, match="bounded wait") as e:
        plan.check()
    assert e.value.status == capi.RG_ERR_TIMEOUT
    plan.check()  # cleared
    out = torch.empty(64, device=gpu)
    plan.run(prt, out)
    plan.check()
    assert torch.equal(out, ref)


def test_full_size_properties(gpu, algo):
    """Config-2 scale (1e8 particles, 512 bins): additivity over a batched split,
    exact scaling by powers of two, reruns (bit-identical for the fused kernel)."""
    n = 100_000_000
    gen = torch.Generator(device=gpu).manual_seed(0)

    def iso(mag):
        mu = torch.rand(n, device=gpu, generator=gen) * 2 - 1
        ph = torch.rand(n, device=gpu, generator=gen) * (2 * np.pi)
        s = torch.sqrt(1 - mu * mu)
        return [mag * s * torch.cos(ph), mag * s * torch.sin(ph), mag * mu]

    umag = 1.0 / (1.0 - torch.rand(n, device=gpu, generator=gen) * (1 - 1e-4))
    u = iso(umag)
    b = iso(torch.exp(0.5 * torch.randn(n, device=gpu, generator=gen)))
    w = torch.rand(n, device=gpu, generator=gen) + 0.5
    bins = np.logspace(-4, 9, 512).astype(np.float32)
    plan = make_plan(bins, algo=algo)
    plan.reserve(2)
    prt = capi.particles(u, b=b, w=w, n=n)
    full = torch.empty(512, device=gpu)
    plan.run(prt, full)
    plan.check()
    again = torch.empty(512, device=gpu)
    plan.run(prt, again)
    plan.check()
    same(full, again, algo)
    split = torch.empty((2, 512), device=gpu)
    offs = torch.tensor([0, 37_000_001, n], dtype=torch.int64, device=gpu)
    plan.run_batched(prt, offs, 2, split)
    plan.check()
    f, s = full.double().cpu().numpy(), split.double().sum(0).cpu().numpy()
    assert max_rel(s, f) < 1e-6
    w2 = w * 2.0
    prt2 = capi.particles(u, b=b, w=w2, n=n)
    doubled = torch.empty(512, device=gpu)
    plan.run(prt2, doubled)
    plan.check()
    same(doubled, full * 2, algo)


def host_particles(P):
    """Pinned host copies of a particle set and the rg_particles over them."""
    H = {k: torch.from_numpy(np.ascontiguousarray(v)).pin_memory() for k, v in P.items()}
    prt = capi.host_particles([H["ux"], H["uy"], H["uz"]], b=[H.get("bx"), H.get("by"), H.get("bz")],
                              w=H.get("w"), n=len(P["ux"]))
    return H, prt


@pytest.mark.parametrize("n", [0, 1, 513, 4099])
def test_host_streaming_matches_oracle(gpu, oracle_lib, table, n, algo):
    P = particles(max(n, 1), seed=40 + n, bfield="iso", weights=True)
    if n == 0:
        P = {k: v[:0] for k, v in P.items()}
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    H, prt = host_particles(P)
    plan = make_plan(bins, algo=algo)
    out = torch.full((200,), -1.0, device=gpu)
    plan.run_host(prt, out)
    plan.check()
    got = out.cpu().numpy()
    truth = oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table) if n else np.zeros(200)
    assert max_rel(got, truth) <= SPECTRUM_RTOL
    assert np.all(got[truth == 0] == 0)


def test_host_streaming_chunks_across_plans(gpu, oracle_lib, algo):
    """Host-resident inputs of several 2^22-particle staging chunks, through two plans
    whose calls interleave on the device's staging buffers, match the same inputs run
    resident on the device; a rerun is bit-identical."""
    sizes = [(1 << 22) + 777, 3 * (1 << 21) + 5, 1000]
    eps = [1.0, 1.0 / 1836.0, 1.0]
    bins = oracle_lib.logspace(1e-4, 1e9, 512)
    plans = [make_plan(bins, 1.0, 1.0, e, algo) for e in eps[:2]]
    sets = [particles(n, seed=90 + i, bfield="iso", weights=True, umax=1e4, index=-2.2)
            for i, n in enumerate(sizes)]
    hosts = [host_particles(P) for P in sets]
    outs = torch.full((3, 512), -1.0, device=gpu)
    for i in range(3):
        plans[i % 2].run_host(hosts[i][1], outs[i])
    for p in plans:
        p.check()
    first = outs.clone()
    for i in range(3):
        plans[i % 2].run_host(hosts[i][1], outs[i])
    same(outs, first, algo)
    for i, P in enumerate(sets):
        T, prt = to_device(P, gpu)
        res = torch.empty(512, device=gpu)
        plans[i % 2].run(prt, res)
        plans[i % 2].check()
        # same items and warps; only the FP64 order of the block partials differs
        assert max_rel(first[i].double().cpu().numpy(), res.double().cpu().numpy()) <= 1e-6


def test_host_streaming_pageable_memory(gpu, oracle_lib, table, algo):
    """Pageable (not pinned) host arrays go through the same call; the result equals the
    pinned-input result bit for bit."""
    P = particles(5000, seed=77, bfield="iso", weights=True)
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    plan = make_plan(bins, algo=algo)
    A = {k: np.ascontiguousarray(v) for k, v in P.items()}
    prt = capi.host_particles([A["ux"], A["uy"], A["uz"]], b=[A["bx"], A["by"], A["bz"]], w=A["w"], n=5000)
    out = torch.empty(200, device=gpu)
    plan.run_host(prt, out)
    plan.check()
    H, hprt = host_particles(P)
    out2 = torch.empty(200, device=gpu)
    plan.run_host(hprt, out2)
    plan.check()
    same(out, out2, algo)
    assert max_rel(out.cpu().numpy(), oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table)) <= SPECTRUM_RTOL


def test_more_than_2_pow_31_particles(gpu, algo):
    """2^31 + 777 particles (u and B each one 8.6 GB stream used for all three components):
    64-bit particle and item indexing; one launch equals the sum of a two-segment batch."""
    n = (1 << 31) + 777
    gen = torch.Generator(device=gpu).manual_seed(12)
    u = torch.rand(n, device=gpu, generator=gen) * 30 + 0.5
    b = torch.rand(n, device=gpu, generator=gen) + 0.2
    prt = capi.particles([u, u, u], b=[b, -b, b], n=n)
    bins = np.logspace(-2, 6, 32).astype(np.float32)
    plan = make_plan(bins, algo=algo)
    plan.reserve(2)
    full = torch.empty(32, device=gpu)
    plan.run(prt, full)
    plan.check()
    split = torch.empty((2, 32), device=gpu)
    offs = torch.tensor([0, (1 << 30) + 3, n], dtype=torch.int64, device=gpu)
    plan.run_batched(prt, offs, 2, split)
    plan.check()
    f, s = full.double().cpu().numpy(), split.double().sum(0).cpu().numpy()
    del u, b
    torch.cuda.empty_cache()
    assert np.all(np.isfinite(f)) and f.max() > 0
    assert max_rel(s, f) < 1e-6


def test_nan_particles_add_nothing(gpu, oracle_lib, table, algo):
    """A NaN momentum or field gives a NaN peak energy, which the reference's e_peak > 0
    test skips (synchrotron.hpp:162); such particles add nothing here either."""
    n = 3000
    P = particles(n, seed=15, bfield="iso")
    P["ux"][:100] = np.nan
    P["bz"][100:200] = np.nan
    bins = oracle_lib.logspace(0.01, 1e7, 200)
    got = gpu_spectrum(P, bins, gpu, algo=algo)
    assert np.all(np.isfinite(got))
    only = oracle_lib.sync_spectrum_f64({k: v[200:] for k, v in P.items()}, bins, 1.0, 1.0, 1.0, table)
    assert max_rel(got, only) <= SPECTRUM_RTOL


def test_host_streaming_from_two_threads(gpu, oracle_lib, algo):
    """Two host threads, each with its own plan and stream, stream host-resident particles
    through the device's shared staging buffers at the same time; each result equals the
    same call made alone."""
    import threading  # noqa: PLC0415

    bins = oracle_lib.logspace(1e-4, 1e9, 256)
    sets = [particles((1 << 22) + 1000 * i, seed=60 + i, bfield="iso", weights=True) for i in range(2)]
    hosts = [host_particles(P) for P in sets]
    plans = [make_plan(bins, 1.0, 1.0, 1.0, algo), make_plan(bins, 1.0, 1.0, 0.5, algo)]
    alone = []
    for i in range(2):
        o = torch.empty(256, device=gpu)
        plans[i].run_host(hosts[i][1], o)
        plans[i].check()
        alone.append(o.cpu())
    outs = [torch.empty(256, device=gpu) for _ in range(2)]
    streams = [torch.cuda.Stream(gpu) for _ in range(2)]
    errors = []

    def worker(i):
        try:
            for _ in range(3):
                plans[i].run_host(hosts[i][1], outs[i], streams[i].cuda_stream)
            streams[i].synchronize()
        except Exception as e:  # noqa: BLE001
            errors.append(e)

    threads = [threading.Thread(target=worker, args=(i,)) for i in range(2)]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    assert not errors
    for i in range(2):
        plans[i].check(streams[i].cuda_stream)
        same(outs[i].cpu(), alone[i], algo)

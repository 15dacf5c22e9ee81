"""The multi-rank path on the CPU: two gloo ranks split a particle set and a
batched job the way one-process-per-GPU runs split them, each computes its
share with the FP64 oracle (the stand-in for one GPU's kernel), and the one
exchange -- the FP64 sum of the per-rank spectra -- and the max-over-ranks
timing reproduce the single-process results."""

from __future__ import annotations

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
shard = pytest.importorskip("ragnar_gb300.shard")


def test_shard_range_covers_once():
    for n in (0, 1, 7, 1000, 10**9 + 7):
        for world in (1, 2, 3, 8):
            spans = [shard.shard_range(n, r, world) for r in range(world)]
            assert spans[0][0] == 0 and spans[-1][1] == n
            assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
            sizes = [hi - lo for lo, hi in spans]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard.shard_range(10, 2, 2)


def test_shard_segments_whole_and_balanced():
    rng = np.random.default_rng(3)
    counts = np.floor(10 ** rng.uniform(4, 7, 256)).astype(np.int64)
    offs = np.concatenate([[0], np.cumsum(counts)]).tolist()
    for world in (1, 2, 4, 8):
        spans = [shard.shard_segments(offs, r, world) for r in range(world)]
        assert spans[0][0] == 0 and spans[-1][1] == 256
        assert all(a[1] == b[0] for a, b in zip(spans, spans[1:]))
        loads = [offs[s1] - offs[s0] for s0, s1 in spans]
        assert max(loads) <= offs[-1] / world + counts.max()
    with pytest.raises(ValueError):
        shard.shard_segments([0, 5, 3], 0, 2)
    empty = [shard.shard_segments([0, 0, 0], r, 2) for r in range(2)]
    assert empty[0][0] == 0 and empty[0][1] == empty[1][0] and empty[1][1] == 2


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, result_dir):
    import torch.distributed as dist  # noqa: PLC0415

    import oracle  # noqa: PLC0415
    from helpers import particles  # noqa: PLC0415

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        table = oracle.tabulate_ffunc()
        bins = oracle.logspace(0.01, 1e7, 128)
        P = particles(30001, seed=77, bfield="iso", weights=True)
        lo, hi = shard.shard_range(len(P["ux"]), rank, world)
        mine = {k: v[lo:hi] for k, v in P.items()}
        local = oracle.sync_spectrum_f64(mine, bins, 1.0, 1.0, 1.0, table, nthreads=1)
        total = shard.sum_over_ranks(torch.from_numpy(local))
        # batched: whole segments per rank
        offs = [0, 1000, 1000, 9000, 20000, 20001, 30001]
        s0, s1 = shard.shard_segments(offs, rank, world)
        seg = np.zeros((6, 128))
        if s1 > s0:
            a, b = offs[s0], offs[s1]
            part = {k: v[a:b] for k, v in P.items()}
            sub = np.array(offs[s0:s1 + 1], np.int64) - a
            seg[s0:s1] = oracle.sync_spectrum_batched_f64(part, sub, bins, 1.0, 1.0, 1.0, table, nthreads=1)
        segs = shard.sum_over_ranks(torch.from_numpy(seg))
        tmax = shard.max_over_ranks(float(rank + 1))
        np.savez(os.path.join(result_dir, f"rank{rank}.npz"), total=total.numpy(), segs=segs.numpy(), tmax=tmax)
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reproduce_single_process(tmp_path, oracle_lib):
    import torch.multiprocessing as mp  # noqa: PLC0415

    from helpers import particles  # noqa: PLC0415

    world, port = 2, _free_port()
    mp.start_processes(_rank_main, args=(world, port, str(tmp_path)), nprocs=world, start_method="spawn")
    table = oracle_lib.tabulate_ffunc()
    bins = oracle_lib.logspace(0.01, 1e7, 128)
    P = particles(30001, seed=77, bfield="iso", weights=True)
    whole = oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table, nthreads=1)
    offs = np.array([0, 1000, 1000, 9000, 20000, 20001, 30001], np.int64)
    batched = oracle_lib.sync_spectrum_batched_f64(P, offs, bins, 1.0, 1.0, 1.0, table, nthreads=1)
    for r in range(world):
        out = np.load(tmp_path / f"rank{r}.npz")
        np.testing.assert_allclose(out["total"], whole, rtol=1e-12, atol=0)
        np.testing.assert_allclose(out["segs"], batched, rtol=1e-12, atol=0)
        assert float(out["tmax"]) == world

"""Splitting a spectrum job over ranks (one process per GPU).

A particle spectrum is a sum over particles, so the work shards with no data
exchange: each rank computes the spectrum of its own particles (or of its own
segments of a batched job) and, only if one combined spectrum is wanted, the
per-rank spectra are summed once at the end (at most nseg x nbins values).
`torch.distributed` carries that one sum and the timing maximum; it works with
gloo (CPU tensors) and NCCL (CUDA tensors) alike.
"""

from __future__ import annotations

from bisect import bisect_left


def shard_range(n: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous particle range [lo, hi) of `rank`; sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world or n < 0:
        raise ValueError("need n >= 0 and 0 <= rank < world")
    return n * rank // world, n * (rank + 1) // world


def shard_segments(offsets, rank: int, world: int) -> tuple[int, int]:
    """Whole segments [s0, s1) of a batched job for `rank`, balanced by particle
    count: rank r takes the segments whose first particle falls in the r-th
    contiguous share of the particles.  `offsets` is the host list of nseg + 1
    non-decreasing particle offsets."""
    offs = [int(v) for v in offsets]
    if len(offs) < 1 or any(b < a for a, b in zip(offs, offs[1:])):
        raise ValueError("offsets must be a non-decreasing list of nseg + 1 values")
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    nseg, total = len(offs) - 1, offs[-1] - offs[0]

    def first_segment(r):
        if r >= world:
            return nseg
        target = offs[0] + total * r // world
        return min(bisect_left(offs, target, 0, nseg), nseg)

    s0 = 0 if rank == 0 else first_segment(rank)
    s1 = first_segment(rank + 1)
    return s0, max(s0, s1)


def sum_over_ranks(spectrum, group=None):
    """FP64 sum of every rank's spectrum tensor (returned on the input's device)."""
    import torch  # noqa: PLC0415
    import torch.distributed as dist  # noqa: PLC0415

    acc = spectrum.detach().to(torch.float64).clone()
    dist.all_reduce(acc, op=dist.ReduceOp.SUM, group=group)
    return acc


def max_over_ranks(value: float, device=None, group=None) -> float:
    """Largest `value` over the ranks (the job's time is its slowest rank's)."""
    import torch  # noqa: PLC0415
    import torch.distributed as dist  # noqa: PLC0415

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(t.item())

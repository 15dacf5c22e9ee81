"""The allocation-free spectrum entry point, called through the C ABI.

rg_synchrotron_spectrum_noalloc serves callers that cannot allocate device
memory after start-up (a process that hands its whole device memory budget out
up front, or a plugin loaded into one): all of its scratch lives in one fixed
device array inside the library.  Two calls in a row with different particle
sets and photon bins must each match the FP64 oracle and the allocating entry
point (rg_synchrotron_spectrum) within the spectrum tolerance of the other
tests, so a second call cannot be fed by what the first left in the shared
array; and once the library is initialised, further calls must leave the
device's free memory unchanged.  This file is collected last so a stop at the
first failure has run everything else.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from helpers import SPECTRUM_RTOL, max_rel, particles

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
capi = pytest.importorskip("ragnar_gb300.capi")


def _call(fn, prt, bins, out, B0=1.0, g=1.0, eps=1.0):
    capi.check(fn(ctypes.byref(prt), bins.ctypes.data, len(bins), B0, g, eps, out.data_ptr(), 0))


def _run(fn, prt, bins, dev, B0=1.0, g=1.0, eps=1.0):
    out = torch.full((len(bins),), -1.0, device=dev)
    _call(fn, prt, bins, out, B0, g, eps)
    torch.cuda.synchronize()
    return out.cpu().numpy()


def _device_particles(P, dev):
    T = {k: torch.from_numpy(v).to(dev) for k, v in P.items()}
    prt = capi.particles([T["ux"], T["uy"], T["uz"]], b=[T["bx"], T["by"], T["bz"]],
                         e=[T["ex"], T["ey"], T["ez"]] if "ex" in T else None, w=T.get("w"))
    return T, prt


def test_noalloc_matches_oracle_and_allocating_entry_point_twice(gpu, oracle_lib):
    L = capi.lib()
    table = oracle_lib.tabulate_ffunc()
    cases = [
        (particles(70001, seed=91, bfield="iso", weights=True), oracle_lib.logspace(1e-2, 1e7, 200), (1.0, 1.0, 1.0)),
        (particles(30000, seed=92, bfield="z", efield=True), oracle_lib.logspace(1e-4, 1e9, 512), (0.7, 1.3, 2.0)),
    ]
    for P, bins, (B0, g, eps) in cases:
        T, prt = _device_particles(P, gpu)
        got = _run(L.rg_synchrotron_spectrum_noalloc, prt, bins, gpu, B0, g, eps)
        want = _run(L.rg_synchrotron_spectrum, prt, bins, gpu, B0, g, eps)
        truth = oracle_lib.sync_spectrum_f64(P, bins, B0, g, eps, table)
        assert np.all(np.isfinite(got))
        assert max_rel(got, truth) <= SPECTRUM_RTOL
        assert max_rel(got, want) <= SPECTRUM_RTOL
        assert np.array_equal(got == 0, want == 0)


def test_noalloc_calls_leave_free_device_memory_unchanged(gpu):
    P = particles(50000, seed=93, bfield="iso", weights=True)
    T, prt = _device_particles(P, gpu)
    bins = np.logspace(-3, 8, 300).astype(np.float32)
    out = torch.empty(300, device=gpu)
    fn = capi.lib().rg_synchrotron_spectrum_noalloc
    _call(fn, prt, bins, out)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(gpu)
    for _ in range(2):
        _call(fn, prt, bins, out)
        torch.cuda.synchronize()
        assert torch.cuda.mem_get_info(gpu)[0] == free0
    assert bool(torch.isfinite(out).all())


def test_noalloc_zero_bins_is_a_no_op(gpu):
    P = particles(100, seed=2)
    T, prt = _device_particles(P, gpu)
    status = capi.lib().rg_synchrotron_spectrum_noalloc(ctypes.byref(prt), None, 0, 1.0, 1.0, 1.0, None, 0)
    assert status == capi.RG_OK


def test_noalloc_rejects_too_many_bins(gpu):
    P = particles(100, seed=1)
    T, prt = _device_particles(P, gpu)
    bins = np.logspace(-2, 7, 513).astype(np.float32)
    out = torch.empty(513, device=gpu)
    status = capi.lib().rg_synchrotron_spectrum_noalloc(ctypes.byref(prt), bins.ctypes.data, 513, 1.0, 1.0,
                                                        1.0, out.data_ptr(), 0)
    assert status == capi.RG_ERR_ARGUMENT
    assert "512" in capi.lib().rg_last_error().decode()

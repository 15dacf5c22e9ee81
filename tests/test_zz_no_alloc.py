"""The allocation-free spectrum entry point, called through the C ABI.

rg_synchrotron_spectrum_noalloc serves callers that cannot allocate device
memory after start-up (a process that hands its whole device memory budget out
up front, or a plugin loaded into one): all of its scratch lives in one fixed
device array inside the library.  Two calls in a row with different particle
sets and photon bins must each match the allocating entry point
(rg_synchrotron_spectrum) within the spectrum tolerance of the other tests, so a
second call cannot be fed by what the first left in the shared array.  This file
is collected last so a stop at the first failure has run everything else.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from helpers import SPECTRUM_RTOL, max_rel, particles

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")
capi = pytest.importorskip("ragnar_gb300.capi")


def _run(fn, prt, bins, dev, B0=1.0, g=1.0, eps=1.0):
    out = torch.full((len(bins),), -1.0, device=dev)
    capi.check(fn(ctypes.byref(prt), bins.ctypes.data, len(bins), B0, g, eps, out.data_ptr(), 0))
    torch.cuda.synchronize()
    return out.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice(gpu):
    L = capi.lib()
    cases = [
        (particles(70001, seed=91, bfield="iso", weights=True), np.logspace(-2, 7, 200), (1.0, 1.0, 1.0)),
        (particles(30000, seed=92, bfield="z", efield=True), np.logspace(-4, 9, 512), (0.7, 1.3, 2.0)),
    ]
    for P, bins, (B0, g, eps) in cases:
        bins = bins.astype(np.float32)
        T = {k: torch.from_numpy(v).to(gpu) for k, v in P.items()}
        prt = capi.particles([T["ux"], T["uy"], T["uz"]], b=[T["bx"], T["by"], T["bz"]],
                             e=[T["ex"], T["ey"], T["ez"]] if "ex" in T else None, w=T.get("w"))
        want = _run(L.rg_synchrotron_spectrum, prt, bins, gpu, B0, g, eps)
        got = _run(L.rg_synchrotron_spectrum_noalloc, prt, bins, gpu, B0, g, eps)
        assert np.all(np.isfinite(got))
        assert max_rel(got, want) <= SPECTRUM_RTOL
        assert np.array_equal(got == 0, want == 0)


def test_noalloc_rejects_too_many_bins(gpu):
    P = particles(100, seed=1)
    T = {k: torch.from_numpy(v).to(gpu) for k, v in P.items()}
    prt = capi.particles([T["ux"], T["uy"], T["uz"]], b=[T["bx"], T["by"], T["bz"]])
    bins = np.logspace(-2, 7, 513).astype(np.float32)
    out = torch.empty(513, device=gpu)
    status = capi.lib().rg_synchrotron_spectrum_noalloc(ctypes.byref(prt), bins.ctypes.data, 513, 1.0, 1.0,
                                                        1.0, out.data_ptr(), 0)
    assert status == capi.RG_ERR_ARGUMENT
    assert "512" in capi.lib().rg_last_error().decode()

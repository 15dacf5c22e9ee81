"""CPU-side checks of the C ABI library and the drop-in module: every symbol the
header declares is exported, the host-side logic (grids, histogram thresholds,
FP64 quadratures, argument validation) is exact, and the module exposes the
reference's API names.  Nothing here launches a kernel.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest

from helpers import golden

capi = pytest.importorskip("ragnar_gb300.capi")


def test_library_exports_every_header_symbol():
    L = ctypes.CDLL(capi.LIB_PATH)
    names = capi.header_functions()
    assert len(names) >= 25
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, f"declared in include/ragnar_gb300.h but not exported: {missing}"


def test_host_grids_bit_exact_vs_reference():
    L = capi.lib()
    g = golden("grids")
    for key in g.files:
        if key.endswith("_args"):
            continue
        a, b, n = g[key + "_args"]
        out = np.empty(int(n), np.float32)
        fn = L.rg_logspace if key.startswith("log") else L.rg_linspace
        capi.check(fn(float(a), float(b), int(n), out.ctypes.data))
        np.testing.assert_array_equal(out, g[key], err_msg=key)


@pytest.mark.parametrize("args,msg", [
    ((-1.0, 10.0, 5), "Logspace start and stop must be strictly positive"),
    ((10.0, 1.0, 5), "Logspace start must be < stop"),
])
def test_logspace_errors_match_reference(args, msg):
    out = np.empty(8, np.float32)
    with pytest.raises(capi.RgError, match=msg):
        capi.check(capi.lib().rg_logspace(*args, out.ctypes.data))


def test_linspace_error_matches_reference():
    out = np.empty(8, np.float32)
    with pytest.raises(capi.RgError, match="Linspace start must be < stop"):
        capi.check(capi.lib().rg_linspace(3.0, 1.0, 4, out.ctypes.data))


def _thresholds(bins, fourvel):
    bins = np.ascontiguousarray(bins, np.float32)
    thr = np.empty(len(bins), np.float32)
    nan_idx = ctypes.c_int32()
    capi.check(capi.lib().rg_energy_thresholds(bins.ctypes.data, len(bins), int(fourvel),
                                                thr.ctypes.data, ctypes.byref(nan_idx)))
    return thr, nan_idx.value


@pytest.mark.parametrize("case", range(4))
def test_histogram_thresholds_reproduce_reference_index(oracle_lib, case):
    """Bin index from the thresholds == the reference's double expression, for
    random |u|^2 and for the floats on both sides of every threshold."""
    g = golden("histogram")
    bins = g[f"case{case}_bins"]
    _, fourvel = g[f"case{case}_meta"]
    thr, _ = _thresholds(bins, fourvel)
    n = len(bins)
    emin, emax = float(bins.min()), float(bins.max())
    assert thr[0] == 0 and np.all(np.diff(thr) >= 0)

    def idx_from_thr(U):
        return int(np.searchsorted(thr, U, side="right") - 1)

    rng = np.random.default_rng(case)
    samples = list((10.0 ** rng.uniform(-6, 7, 3000)).astype(np.float32))
    for t in thr[1:]:
        if np.isfinite(t):
            samples += [np.nextafter(t, np.float32(0)), t, np.nextafter(t, np.float32(np.inf))]
    samples += [np.float32(0), np.float32(np.inf)]
    for U in samples:
        assert idx_from_thr(U) == oracle_lib.energy_bin_index_usqr(float(U), fourvel, emin, emax, n), U


def test_bessel_and_exact_F_quadratures():
    sp = pytest.importorskip("scipy.special")
    L = capi.lib()
    for x in [1e-6, 1e-4, 1e-2, 0.29, 1.0, 5.0, 20.0, 80.0, 300.0]:
        assert abs(L.rg_debug_bessel_k53(x) / sp.kv(5.0 / 3.0, x) - 1) < 1e-13
    # F(x) = x int_x^inf K_{5/3}: small-x asymptote and a direct quadrature
    x = 1e-8
    asym = 4 * np.pi / (np.sqrt(3) * sp.gamma(1 / 3)) * (x / 2) ** (1 / 3)
    assert abs(L.rg_debug_exact_F(x) / asym - 1) < 1e-4
    si = pytest.importorskip("scipy.integrate")
    for x in [1e-3, 0.29, 1.0, 5.0, 20.0]:
        ref = x * si.quad(lambda t: sp.kv(5.0 / 3.0, t), x, np.inf, limit=400, epsabs=0.0,
                          epsrel=1e-13)[0]
        assert abs(L.rg_debug_exact_F(x) / ref - 1) < 1e-11


REFERENCE_NAMES = [
    # pyinterface.cpp:26-91 and the pyDefine* functions it calls (synchrotron path)
    "Initialize", "Finalize", "EnergyUnits", "Linspace", "Logspace", "Array1D_i", "Array1D_f",
    "Array1D_d", "Bins", "Linbins", "Logbins", "TabulatedFunction", "TabulatedFunction_log",
    "PlawGenerator", "BrokenPlawGenerator", "DeltaGenerator", "TabulatedDistribution",
    "Particles_1D", "Particles_2D", "Particles_3D", "SynchrotronSpectrum_1D",
    "SynchrotronSpectrum_2D", "SynchrotronSpectrum_3D", "SynchrotronSpectrumFromDist",
    "Ffunc_integrand", "ICSpectrum",
]


def test_module_exposes_reference_api():
    rg = pytest.importorskip("ragnar_gb300")
    missing = [n for n in REFERENCE_NAMES if not hasattr(rg, n)]
    assert not missing, missing
    for cls in ("Particles_1D", "Particles_2D", "Particles_3D"):
        c = getattr(rg, cls)
        for meth in ("fromArrays", "setNactive", "setIgnoreCoords", "allocate", "printHead",
                     "is_allocated", "nactive", "nalloc", "label", "energyDistribution", "X", "U",
                     "E", "B", "__len__", "__repr__"):
            assert hasattr(c, meth), (cls, meth)
    for cls, meths in (("Array1D_i", ("as_array", "extent", "head", "__repr__")),
                       ("Array1D_f", ("as_array", "extent", "head", "__repr__")),
                       ("Array1D_d", ("as_array", "extent", "head", "__repr__")),
                       ("Bins", ("log_spaced", "unit")),
                       ("TabulatedDistribution", ("extent", "log_spaced", "EnergyBins", "F")),
                       ("PlawGenerator", ("compute",)), ("BrokenPlawGenerator", ("compute",)),
                       ("DeltaGenerator", ("compute",))):
        for meth in meths:
            assert hasattr(getattr(rg, cls), meth), (cls, meth)
    assert rg.EnergyUnits.mec2 == "mec2" and rg.EnergyUnits.mpc2 == "mpc2"
    p = rg.Particles_3D("electrons")
    assert p.label() == "electrons" and not p.is_allocated() and len(p) == 0


def test_particle_structs_keep_their_arrays():
    """rg_particles holds raw addresses: the Python structure keeps the arrays it was built
    from alive, so temporaries passed to particles() / host_particles() are not freed (and
    their memory reused by later allocations) while the structure is in use."""
    import gc  # noqa: PLC0415
    import weakref  # noqa: PLC0415

    torch = pytest.importorskip("torch")
    t = torch.ones(8)
    ref = weakref.ref(t)
    p = capi.particles([t, t, t], b=[None, None, torch.zeros(8)])
    del t
    gc.collect()
    assert ref() is not None and p.u[0] == ref().data_ptr()
    del p
    gc.collect()
    assert ref() is None

    a = np.ones(8, np.float32)
    ref = weakref.ref(a)
    h = capi.host_particles([a, a, a])
    del a
    gc.collect()
    assert ref() is not None and h.u[0] == ref().ctypes.data


def test_placed_entry_points_reject_bad_arguments():
    """The placed forward and adjoint check their arguments before any device work: no plan,
    no placement buffer or no gradient input is RG_ERR_ARGUMENT with a message."""
    L = capi.lib()
    p = capi.particles([16, 32, 48], n=4)  # addresses only; nothing is read
    assert L.rg_spectrum_run_placed(None, ctypes.byref(p), 8, 8, None) == capi.RG_ERR_ARGUMENT
    assert b"rg_spectrum_run_placed" in L.rg_last_error()
    assert L.rg_spectrum_adjoint_placed(None, ctypes.byref(p), 8, 8, None, None, None, None,
                                        None) == capi.RG_ERR_ARGUMENT
    assert b"rg_spectrum_adjoint_placed" in L.rg_last_error()

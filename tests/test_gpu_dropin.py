"""The reference's test suite (src/tests/*.py) restated against the drop-in
module: same calls, same assertions, plus exact checks against the reference's
outputs (golden fixtures) and the reference's error behaviour."""

from __future__ import annotations

import numpy as np
import pytest

from helpers import golden, max_rel, slope

pytestmark = pytest.mark.gpu

rg = pytest.importorskip("ragnar_gb300")


@pytest.fixture(scope="module", autouse=True)
def init():
    rg.Initialize()
    rg.SetVerbose(False)
    yield


def check_slope(xs, ys, p, xmin, xmax, atol=1e-2):
    return np.isclose(p, slope(xs, ys, xmin, xmax), atol=atol)


# --- arrays_bins.py ----------------------------------------------------------------
def test_arrays_bins():
    array = np.arange(123)
    assert np.all(np.isclose(rg.Array1D_i(array.astype(np.int32)).as_array(), array))
    assert np.all(np.isclose(rg.Array1D_f(array.astype(np.float32)).as_array(), array))
    assert np.all(np.isclose(rg.Array1D_d(array.astype(np.float64)).as_array(), array))
    assert rg.Array1D_d(array.astype(np.float64)).extent() == 123
    bins = rg.Bins(np.logspace(-2.5, 2.5, 213))
    bins.log_spaced = True
    bins.unit = rg.EnergyUnits.mec2
    assert bins.unit == rg.EnergyUnits.mec2 and bins.extent() == 213 and bins.log_spaced
    assert repr(rg.Array1D_f(np.ones(5, np.float32))) == "1D Array [ size: 5 ]"


# --- linspace_logspace.py ----------------------------------------------------------
def test_linspace_logspace():
    assert np.all(np.isclose(rg.Linspace(-32.0, 4832.0, 56).as_array(), np.linspace(-32.0, 4832.0, 56)))
    assert np.all(np.isclose(rg.Logspace(10**-2.5, 10**2.5, 213).as_array(), np.logspace(-2.5, 2.5, 213)))
    lb = rg.Linbins(55.0, 56.0, 123)
    assert np.all(np.isclose(lb.as_array(), np.linspace(55.0, 56.0, 123))) and not lb.log_spaced
    gb = rg.Logbins(1, 1e3, 22)
    assert np.all(np.isclose(gb.as_array(), np.logspace(0, 3, 22))) and gb.log_spaced
    # bit-exact against the reference's own grids
    g = golden("grids")
    for key in g.files:
        if key.endswith("_args"):
            continue
        a, b, n = g[key + "_args"]
        fn = rg.Logspace if key.startswith("log") else rg.Linspace
        np.testing.assert_array_equal(fn(float(a), float(b), int(n)).as_array(), g[key])
    with pytest.raises(RuntimeError, match="Logspace start must be < stop"):
        rg.Logspace(10.0, 1.0, 5)


# --- distributions.py --------------------------------------------------------------
def test_distributions():
    for norm in (rg.Logspace, rg.Linspace):
        d = rg.TabulatedDistribution(rg.Bins(norm(1e-2, 1, int(1e6))), rg.DeltaGenerator(2e-2, 0.01))
        assert np.isclose(np.trapezoid(d.F().as_array(), d.EnergyBins().as_array()), 1)
    for norm in (rg.Logspace, rg.Linspace):
        d = rg.TabulatedDistribution(rg.Bins(norm(1e-3, 10, int(1e6))),
                                     rg.BrokenPlawGenerator(0.3, 0.23, -1.0, 1e-2, 2))
        assert np.isclose(np.trapezoid(d.F().as_array(), d.EnergyBins().as_array()), 1)
    for norm in (rg.Logspace, rg.Linspace):
        d = rg.TabulatedDistribution(rg.Bins(norm(1e-2, 1, int(1e6))), rg.PlawGenerator(-1.2, 1e-2, 1))
        assert np.isclose(np.trapezoid(d.F().as_array(), d.EnergyBins().as_array()), 1)


def test_generators_bit_exact():
    g = golden("generators")
    bins = rg.Bins(g["bins"])
    np.testing.assert_array_equal(rg.PlawGenerator(-1.2, 1e-2, 1.0).compute(bins).as_array(), g["plaw"])
    np.testing.assert_array_equal(rg.PlawGenerator(-2.5, 0.5, 0.0).compute(bins).as_array(), g["plaw_open"])
    np.testing.assert_array_equal(rg.PlawGenerator(-1.0, 0.1, 5.0).compute(bins).as_array(), g["plaw_m1"])
    np.testing.assert_array_equal(rg.BrokenPlawGenerator(0.3, 0.23, -1.0, 1e-2, 2.0).compute(bins).as_array(),
                                  g["bplaw"])
    np.testing.assert_array_equal(rg.BrokenPlawGenerator(0.3, 0.5, -2.5, 1e-2, 0.0).compute(bins).as_array(),
                                  g["bplaw_open"])
    np.testing.assert_array_equal(rg.DeltaGenerator(2e-2, 0.01).compute(bins).as_array(), g["delta"])
    with pytest.raises(RuntimeError, match="normalization diverges"):
        rg.PlawGenerator(-1.5)
    with pytest.raises(RuntimeError, match="e_extent|extent"):
        rg.TabulatedDistribution(rg.Logbins(1, 10, 5), rg.Array1D_f(np.ones(4, np.float32)))


# --- particles.py -------------------------------------------------------------------
KEYS = ["U1", "U3", "E1", "E2", "E3", "B1", "B2", "B3"]


def _arrays(rng, n=10):
    return {k: rng.random(n) for k in KEYS}


def _getters(p):
    return [p.U(1), p.U(3), p.E(1), p.E(2), p.E(3), p.B(1), p.B(2), p.B(3)]


def test_prtls():
    prtls = rg.Particles_3D("electrons")
    assert prtls.label() == "electrons" and not prtls.is_allocated()
    rng = np.random.default_rng(123)
    a = _arrays(rng)
    prtls.fromArrays(a)
    for k, f in zip(KEYS, _getters(prtls)):
        assert np.all(np.isclose(a[k], f.as_array()))
    assert prtls.is_allocated() and prtls.nactive() == 10 and prtls.nalloc() == 10
    b = _arrays(rng)
    prtls.fromArrays(b, append=True)
    for k, f in zip(KEYS, _getters(prtls)):
        assert np.all(np.isclose(a[k], f.as_array()[:10]))
        assert np.all(np.isclose(b[k], f.as_array()[10:]))
    assert prtls.nactive() == 20 and prtls.nalloc() == 20
    with pytest.raises(RuntimeError, match="append = True"):
        prtls.fromArrays(b)


def test_prtls_preallocated():
    rng = np.random.default_rng(123)
    prtls = rg.Particles_3D("electrons")
    prtls.allocate(20)
    assert prtls.nactive() == 0 and prtls.nalloc() == 20
    a = _arrays(rng)
    prtls.fromArrays(a, append=True)
    assert prtls.nactive() == 10 and prtls.nalloc() == 20
    for k, f in zip(KEYS, _getters(prtls)):
        assert np.all(np.isclose(a[k], f.as_array()))
    b = _arrays(rng)
    prtls.fromArrays(b, append=True)
    assert prtls.nactive() == 20 and prtls.nalloc() == 20
    for k, f in zip(KEYS, _getters(prtls)):
        assert np.all(np.isclose(a[k], f.as_array()[:10]))
        assert np.all(np.isclose(b[k], f.as_array()[10:]))


def test_prtls_coords():
    rng = np.random.default_rng(123)
    prtls = rg.Particles_3D("electrons")
    X1s, U3s = rng.random(10), rng.random(10)
    prtls.fromArrays({"X1": X1s, "U3": U3s}, append=True)
    assert np.all(np.isclose(prtls.X(1).as_array(), X1s))
    assert np.all(np.isclose(prtls.U(3).as_array(), U3s))
    assert np.all(np.isclose(prtls.U(1).as_array(), np.zeros_like(U3s)))
    assert np.all(np.isclose(prtls.E(1).as_array(), np.zeros_like(U3s)))


def test_prtls_errors():
    p = rg.Particles_3D("p")
    with pytest.raises(RuntimeError, match="No particles provided"):
        p.fromArrays({"U1": np.zeros(0, np.float32)})
    with pytest.raises(RuntimeError, match="Inconsistent number of particles"):
        p.fromArrays({"U1": np.zeros(3, np.float32), "U2": np.zeros(4, np.float32)})
    with pytest.raises(RuntimeError, match="not allocated"):
        p.setNactive(3)
    p.fromArrays({"U1": np.ones(3, np.float32)})
    with pytest.raises(IndexError):
        p.U(4)
    p.setIgnoreCoords(True)
    with pytest.raises(RuntimeError, match="coordinates ignored"):
        p.X(1)
    with pytest.raises(RuntimeError, match="already allocated"):
        p.allocate(10)


# --- synchrotron.py -----------------------------------------------------------------
def test_sync_log():
    p = 2.23
    dist = rg.TabulatedDistribution(rg.Logbins(1, 1000, 200), rg.PlawGenerator(-p, 1, 1000))
    bins = rg.Logbins(0.01, 1e7, 200)
    bins.unit = rg.EnergyUnits.mec2
    s = rg.SynchrotronSpectrumFromDist(dist, bins, 1, 1)
    x, y = bins.as_array(), s.as_array()
    assert check_slope(dist.EnergyBins().as_array(), dist.F().as_array(), -p, 2, 800)
    assert check_slope(x, y, -p / 2 + 3 / 2, 10, 1e4)
    assert check_slope(x, y, 1 / 3 + 1, 3e-2, 2e-1, atol=0.1)
    g = golden("fromdist")
    np.testing.assert_array_equal(dist.F().as_array(), g["case0_f"])
    assert max_rel(y, g["case0_ref"]) < 2e-5


def test_sync_lin():
    p = 2.5
    dist = rg.TabulatedDistribution(rg.Linbins(1, 1000, 10000), rg.PlawGenerator(-p, 1, 1000))
    bins = rg.Logbins(0.01, 1e6, 500)
    bins.unit = rg.EnergyUnits.mec2
    s = rg.SynchrotronSpectrumFromDist(dist, bins, 1, 1)
    assert check_slope(dist.EnergyBins().as_array(), dist.F().as_array(), -p, 2, 800)
    assert check_slope(bins.as_array(), s.as_array(), -p / 2 + 3 / 2, 10, 1e4)
    assert check_slope(bins.as_array(), s.as_array(), 1 / 3 + 1, 3e-2, 2e-1, atol=0.1)


def test_sync_prtls():
    rng = np.random.default_rng(123)

    def random_plaw(size, xmin, xmax, p, rng):
        return ((xmax ** (p + 1) - xmin ** (p + 1)) * rng.random(size) + xmin ** (p + 1)) ** (1 / (p + 1))

    n = int(1e5)
    rnd1 = 2 * (rng.random(n) - 0.5)
    rnd2 = 2 * np.pi * rng.random(n)
    prtls = rg.Particles_3D("pairs")
    prtls.fromArrays({"U1": random_plaw(n, 1, 100, -2, rng),
                      "B1": np.sqrt(1 - rnd1**2) * np.cos(rnd2),
                      "B2": np.sqrt(1 - rnd1**2) * np.sin(rnd2),
                      "B3": rnd1})
    dist = prtls.energyDistribution(rg.Logbins(1, 1e3, 100))
    bins = rg.Logbins(0.01, 1e5, 200, rg.EnergyUnits.mec2)
    s = rg.SynchrotronSpectrum_3D(prtls, bins, 1, 1, 1)
    sd = rg.SynchrotronSpectrumFromDist(dist, bins, 1, 1)
    assert np.abs((s.as_array() * 1.3 - sd.as_array()) / sd.as_array()).max() < 0.15


def test_sync_units_required():
    p = rg.Particles_3D("e")
    p.fromArrays({"U1": np.ones(4, np.float32), "B3": np.ones(4, np.float32)})
    with pytest.raises(RuntimeError, match="bins_e_syn must be in units of mc\\^2"):
        rg.SynchrotronSpectrum_3D(p, rg.Logbins(0.01, 1e3, 10), 1, 1, 1)


def test_spectrum_matches_reference_fixture_and_weights(oracle_lib):
    g = golden("spectrum")
    u, b = g["iso_u"], g["iso_b"]
    p = rg.Particles_3D("iso")
    p.fromArrays({"U1": u[0], "U2": u[1], "U3": u[2], "B1": b[0], "B2": b[1], "B3": b[2]})
    bins = rg.Bins(g["iso_bins"], rg.EnergyUnits.mec2)
    s = rg.SynchrotronSpectrum_3D(p, bins, 1, 1, 1).as_array()
    table = oracle_lib.tabulate_ffunc()
    P = {"ux": u[0], "uy": u[1], "uz": u[2], "bx": b[0], "by": b[1], "bz": b[2]}
    truth = oracle_lib.sync_spectrum_f64(P, g["iso_bins"], 1, 1, 1, table)
    assert max_rel(s, truth) <= 1e-5
    # extension: weights through fromArrays key "W"
    w = np.linspace(0.5, 1.5, u.shape[1]).astype(np.float32)
    pw = rg.Particles_3D("w")
    pw.fromArrays({"U1": u[0], "U2": u[1], "U3": u[2], "B1": b[0], "B2": b[1], "B3": b[2], "W": w})
    sw = rg.SynchrotronSpectrum_3D(pw, bins, 1, 1, 1).as_array()
    assert max_rel(sw, oracle_lib.sync_spectrum_f64(dict(P, w=w), g["iso_bins"], 1, 1, 1, table)) <= 1e-5


def test_energy_distribution_matches_reference_fixture():
    g = golden("histogram")
    u = g["u"]
    p = rg.Particles_3D("h")
    p.fromArrays({"U1": u[0], "U2": u[1], "U3": u[2]})
    for i in range(4):
        bins_arr, (logb, fourvel), F = g[f"case{i}_bins"], g[f"case{i}_meta"], g[f"case{i}_F"]
        bins = rg.Bins(bins_arr)
        bins.log_spaced = bool(logb)
        d = p.energyDistribution(bins, bool(fourvel))
        assert d.log_spaced() == bool(logb) and d.extent() == len(bins_arr)
        if logb:
            m = F > 0
            assert np.max(np.abs(d.F().as_array()[m] - F[m]) / F[m]) < 1e-5
        else:
            np.testing.assert_array_equal(d.F().as_array(), F)


def test_ffunc_integrand_matches_reference():
    g = golden("ftable")
    for x, y in zip(g["xq"][:16], g["yq"][:16]):
        got = np.float32(rg.Ffunc_integrand(float(x)))
        assert abs(got - y) <= 2 * np.spacing(y) or got == y


def test_batched_extension(oracle_lib):
    g = golden("spectrum")
    u, b = g["iso_u"], g["iso_b"]
    p = rg.Particles_3D("iso")
    p.fromArrays({"U1": u[0], "U2": u[1], "U3": u[2], "B1": b[0], "B2": b[1], "B3": b[2]})
    bins = rg.Bins(g["iso_bins"], rg.EnergyUnits.mec2)
    offs = [0, 1000, 1000, 2500]
    S = rg.SynchrotronSpectrumBatched_3D(p, offs, bins, 1, 1, 1)
    assert S.shape == (3, len(g["iso_bins"]))
    table = oracle_lib.tabulate_ffunc()
    P = {"ux": u[0], "uy": u[1], "uz": u[2], "bx": b[0], "by": b[1], "bz": b[2]}
    truth = oracle_lib.sync_spectrum_batched_f64(P, offs, g["iso_bins"], 1, 1, 1, table)
    assert max_rel(S[0], truth[0]) <= 1e-5 and np.all(S[1] == 0) and max_rel(S[2], truth[2]) <= 1e-5

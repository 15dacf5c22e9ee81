"""The assertions of the reference's own tests (src/tests/synchrotron.py), applied
to the oracle.  They pin the oracle's physics to what the reference's test suite
checks: the spectral slopes of a power-law distribution and the agreement of the
particle spectrum with the spectrum of the particles' histogram.
"""

from __future__ import annotations

import numpy as np
import pytest

from helpers import golden, isotropic, powerlaw, slope

pytestmark = pytest.mark.usefixtures("oracle_lib")


@pytest.mark.parametrize("case,p", [(0, 2.23), (1, 2.5)])
def test_fromdist_slopes(oracle_lib, case, p):
    # tests/synchrotron.py:14-59: slope -p/2 + 3/2 on [10, 1e4] (atol 1e-2) and
    # the low-energy 4/3 slope on [3e-2, 2e-1] (atol 0.1)
    g = golden("fromdist")
    gb, f, logb, bins = g[f"case{case}_gb"], g[f"case{case}_f"], bool(g[f"case{case}_log"]), g[f"case{case}_bins"]
    s = oracle_lib.sync_from_dist_f64(gb, f, logb, bins, 1.0, 1.0, oracle_lib.tabulate_ffunc())[0]
    assert abs(slope(gb.astype(np.float64), f.astype(np.float64), 2, 800) + p) < 1e-2
    assert abs(slope(bins.astype(np.float64), s, 10, 1e4) - (-p / 2 + 1.5)) < 1e-2
    assert abs(slope(bins.astype(np.float64), s, 3e-2, 2e-1) - 4.0 / 3.0) < 0.1


def test_particles_vs_distribution(oracle_lib):
    # tests/synchrotron.py:62-104: 1e5 particles with U1 ~ power law p=-2 on [1,100],
    # isotropic unit B; spectrum * 1.3 vs spectrum of the histogram within 15%
    rng = np.random.default_rng(123)
    n = 100000
    rnd1 = 2 * (rng.random(n) - 0.5)
    rnd2 = 2 * np.pi * rng.random(n)
    b1 = (np.sqrt(1 - rnd1**2) * np.cos(rnd2)).astype(np.float32)
    b2 = (np.sqrt(1 - rnd1**2) * np.sin(rnd2)).astype(np.float32)
    b3 = rnd1.astype(np.float32)
    u1 = powerlaw(rng, n, 1.0, 100.0, -2.0).astype(np.float32)
    z = np.zeros(n, np.float32)
    P = {"ux": u1, "uy": z, "uz": z, "bx": b1, "by": b2, "bz": b3}
    table = oracle_lib.tabulate_ffunc()
    hb = oracle_lib.logspace(1.0, 1e3, 100)
    _, h64, _ = oracle_lib.energy_distribution(u1, z, z, hb, True, True)
    bins = oracle_lib.logspace(0.01, 1e5, 200)
    s_p = oracle_lib.sync_spectrum_f64(P, bins, 1.0, 1.0, 1.0, table)
    s_d = oracle_lib.sync_from_dist_f64(hb, h64.astype(np.float32), True, bins, 1.0, 1.0, table)[0]
    assert np.max(np.abs((s_p * 1.3 - s_d) / s_d)) < 0.15


def test_isotropic_helper_is_unit_norm():
    rng = np.random.default_rng(0)
    v = isotropic(rng, 1000, np.ones(1000))
    assert np.allclose(np.sqrt(v[0] ** 2 + v[1] ** 2 + v[2] ** 2), 1.0, atol=1e-6)


def test_ic_slope_and_peak(oracle_lib):
    """The reference's own IC checks (tests/ic.py:15-54), on its configuration: for a
    particle power law of index -p the Thomson-regime slope of E^2 dN/dE is -p/2 + 3/2
    (to 1e-2 between 2e3 and 2e4), and the peak sits at e_break * gamma_max^2 (10 %)."""
    g = golden("ic")
    args = (g["case0_gb"], g["case0_f"], True, g["case0_es"], g["case0_fs"], g["case0_eic"])
    x = g["case0_eic"].astype(np.float64)
    y = oracle_lib.ic_spectrum_f64(*args)
    assert abs(slope(x, y, 2e3, 2e4) - (-1.5 / 2 + 1.5)) < 1e-2
    assert abs(x[np.argmax(y)] / (1e-8 * 1e7**2) - 1.0) < 0.1

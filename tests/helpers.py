"""Shared input generators and comparisons for the tests."""

from __future__ import annotations

import os
import platform

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# relative tolerance of every spectrum against the FP64 oracle, on bins above
# 1e-12 of the peak (the target the synchrotron path is built to)
SPECTRUM_RTOL = 1e-5
PEAK_FLOOR = 1e-12


# The fixtures were generated on x86_64 with 8 OpenMP threads; the reference's
# float math (glibc log10f, pow) is reproduced bit for bit on that platform.
SAME_PLATFORM_AS_FIXTURES = platform.machine() == "x86_64"


def assert_equal_or_close(a, b, rtol=1e-6):
    if SAME_PLATFORM_AS_FIXTURES:
        np.testing.assert_array_equal(a, b)
    else:
        np.testing.assert_allclose(a, b, rtol=rtol, atol=0)


def golden(name: str):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


def isotropic(rng, n, mag):
    mu = rng.uniform(-1.0, 1.0, n)
    ph = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - mu**2)
    return [(mag * s * np.cos(ph)).astype(np.float32), (mag * s * np.sin(ph)).astype(np.float32),
            (mag * mu).astype(np.float32)]


def powerlaw(rng, n, lo, hi, index):
    """|u| with dN/d|u| ~ |u|^index on [lo, hi] by inverse CDF."""
    q = index + 1.0
    if abs(q) < 1e-12:
        return lo * (hi / lo) ** rng.random(n)
    return ((hi**q - lo**q) * rng.random(n) + lo**q) ** (1.0 / q)


def particles(n, seed=0, bfield="z", efield=False, weights=False, umax=100.0, index=-2.0):
    """Seeded particle set as float32 SoA arrays (dict ux..bz[, ex.., w])."""
    rng = np.random.default_rng(seed)
    u = isotropic(rng, n, powerlaw(rng, n, 1.0, umax, index))
    P = {"ux": u[0], "uy": u[1], "uz": u[2]}
    if bfield == "z":
        P.update(bx=np.zeros(n, np.float32), by=np.zeros(n, np.float32), bz=np.ones(n, np.float32))
    else:
        b = isotropic(rng, n, rng.lognormal(0.0, 0.5, n))
        P.update(bx=b[0], by=b[1], bz=b[2])
    if efield:
        e = isotropic(rng, n, 0.3 * rng.random(n))
        P.update(ex=e[0], ey=e[1], ez=e[2])
    if weights:
        P["w"] = rng.uniform(0.5, 1.5, n).astype(np.float32)
    return P


def max_rel(a, ref, floor=PEAK_FLOOR):
    """Max relative error of `a` vs `ref` on bins above floor * peak (0 if none)."""
    a = np.asarray(a, np.float64)
    ref = np.asarray(ref, np.float64)
    if ref.size == 0 or not np.any(ref > 0):
        return 0.0
    m = ref > floor * ref.max()
    return float(np.max(np.abs(a[m] - ref[m]) / ref[m]))


def slope(xs, ys, xmin, xmax):
    m = (xs > xmin) & (xs < xmax)
    p, _ = np.polyfit(np.log10(xs[m]), np.log10(ys[m]), 1)
    return p

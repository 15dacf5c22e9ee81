"""Generates the golden fixtures in tests/golden/ from the reference itself.

The reference library is compiled from its own, unmodified sources against the
Kokkos-API shim (``oracle/build_ref.sh`` -> ``oracle/_ref/``) and imported here
under its own module name; every output below is what the reference's public
API returns for seeded inputs.  Run from the repository root where the
reference tree is present:

    bash oracle/build_ref.sh && OMP_NUM_THREADS=8 python tests/golden/make_golden.py
    OMP_NUM_THREADS=8 python tests/golden/make_golden.py ic     # ic.npz only

The fixtures are small (.npz, a few hundred KB in total) and are committed; the
tests never need the reference tree.
"""

from __future__ import annotations

import glob
import importlib.util
import os
import sys
import zlib

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))


def load_reference():
    cands = glob.glob(os.path.join(ROOT, "oracle", "_ref", "ragnar*.so"))
    if not cands:
        sys.exit("oracle/_ref/ragnar*.so not built (run oracle/build_ref.sh)")
    spec = importlib.util.spec_from_file_location("ragnar", cands[0])
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.Initialize()
    return mod


def isotropic(rng, n, mag):
    mu = rng.uniform(-1.0, 1.0, n)
    ph = rng.uniform(0.0, 2.0 * np.pi, n)
    s = np.sqrt(1.0 - mu**2)
    return [(mag * s * np.cos(ph)).astype(np.float32), (mag * s * np.sin(ph)).astype(np.float32),
            (mag * mu).astype(np.float32)]


def main() -> None:
    rg = load_reference()

    # --- grids (snippets.cpp:21-62) ---------------------------------------------
    grids = {}
    for i, (a, b, n) in enumerate([(1e-6, 100.0, 200), (0.01, 1e7, 200), (1e-4, 1e9, 512),
                                   (10**-2.5, 10**2.5, 213), (1.0, 1e3, 22), (1.0, 1e6, 1024),
                                   (1e-2, 1e13, 1024), (0.37, 0.38, 7)]):
        grids[f"log_{i}_args"] = np.array([a, b, n], np.float64)
        grids[f"log_{i}"] = rg.Logspace(a, b, n).as_array()
    for i, (a, b, n) in enumerate([(-32.0, 4832.0, 56), (55.0, 56.0, 123), (1.0, 1000.0, 10000),
                                   (0.5, 150.0, 100)]):
        grids[f"lin_{i}_args"] = np.array([a, b, n], np.float64)
        grids[f"lin_{i}"] = rg.Linspace(a, b, n).as_array()
    np.savez_compressed(os.path.join(HERE, "grids.npz"), **grids)

    # --- F table (synchrotron.cpp:28-65) ------------------------------------------
    xs = rg.Logspace(1e-6, 100.0, 200).as_array()
    ys = np.array([rg.Ffunc_integrand(float(x)) for x in xs], np.float32)
    ys[xs.astype(np.float64) < 1e-6] = 0.0  # TabulateFfunc's first-node rule (synchrotron.cpp:58)
    rng = np.random.default_rng(101)
    xq = (10.0 ** rng.uniform(-7.0, 1.5, 64)).astype(np.float32)
    yq = np.array([rg.Ffunc_integrand(float(x)) for x in xq], np.float32)
    np.savez_compressed(os.path.join(HERE, "ftable.npz"), x=xs, y=ys, xq=xq, yq=yq)

    # --- particle spectra (synchrotron.cpp:107-145) --------------------------------
    spectra = {}
    cases = [
        # name, n, bins (lo, hi, n), B field, E field
        ("c1", 3000, (0.01, 1e7, 200), "z", False),
        ("iso", 2500, (1e-4, 1e9, 512), "iso", False),
        ("efield", 2000, (0.01, 1e6, 150), "iso", True),
    ]
    for name, n, (lo, hi, nb), bmode, emode in cases:
        rng = np.random.default_rng(zlib.crc32(name.encode()))
        umag = 1.0 / (1.0 - rng.random(n) * (1.0 - 1.0 / 100.0))
        u = isotropic(rng, n, umag)
        if bmode == "z":
            b = [np.zeros(n, np.float32), np.zeros(n, np.float32), np.ones(n, np.float32)]
        else:
            b = isotropic(rng, n, rng.lognormal(0.0, 0.5, n))
        arrays = {"U1": u[0], "U2": u[1], "U3": u[2], "B1": b[0], "B2": b[1], "B3": b[2]}
        e = None
        if emode:
            e = isotropic(rng, n, 0.3 * rng.random(n))
            arrays.update({"E1": e[0], "E2": e[1], "E3": e[2]})
        prt = rg.Particles_3D(name)
        prt.fromArrays(arrays)
        bins = rg.Logbins(lo, hi, nb, rg.EnergyUnits.mec2)
        s = rg.SynchrotronSpectrum_3D(prt, bins, 1.0, 1.0, 1.0).as_array()
        spectra[f"{name}_u"] = np.stack(u)
        spectra[f"{name}_b"] = np.stack(b)
        spectra[f"{name}_e"] = np.stack(e) if e is not None else np.zeros((3, n), np.float32)
        spectra[f"{name}_bins"] = bins.as_array()
        spectra[f"{name}_ref"] = s
    np.savez_compressed(os.path.join(HERE, "spectrum.npz"), **spectra)

    # --- energy distribution (particles.cpp:189-260) -------------------------------
    hist = {}
    rng = np.random.default_rng(7)
    n = 20001
    umag = 1.0 / (1.0 - rng.random(n) * (1.0 - 1.0 / 100.0))
    u = isotropic(rng, n, umag)
    prt = rg.Particles_3D("h")
    prt.fromArrays({"U1": u[0], "U2": u[1], "U3": u[2]})
    hist["u"] = np.stack(u)
    for i, (kind, lo, hi, nb, fourvel) in enumerate([("log", 1e-2, 1e3, 200, True),
                                                      ("log", 1.0, 1e3, 100, False),
                                                      ("lin", 0.5, 150.0, 100, True),
                                                      ("lin", 0.5, 150.0, 77, False)]):
        bins = rg.Logbins(lo, hi, nb) if kind == "log" else rg.Linbins(lo, hi, nb)
        d = prt.energyDistribution(bins, fourvel)
        hist[f"case{i}_bins"] = bins.as_array()
        hist[f"case{i}_meta"] = np.array([kind == "log", fourvel], np.int32)
        hist[f"case{i}_F"] = d.F().as_array()
    np.savez_compressed(os.path.join(HERE, "histogram.npz"), **hist)

    # --- spectrum from a distribution (synchrotron.cpp:69-105) ---------------------
    fd = {}
    for i, (kind, n, p) in enumerate([("log", 200, 2.23), ("lin", 10000, 2.5)]):
        gb = rg.Logbins(1.0, 1000.0, n) if kind == "log" else rg.Linbins(1.0, 1000.0, n)
        dist = rg.TabulatedDistribution(gb, rg.PlawGenerator(-p, 1.0, 1000.0))
        bins = rg.Logbins(0.01, 1e7, 200, rg.EnergyUnits.mec2)
        fd[f"case{i}_gb"] = gb.as_array()
        fd[f"case{i}_f"] = dist.F().as_array()
        fd[f"case{i}_log"] = np.array(kind == "log")
        fd[f"case{i}_bins"] = bins.as_array()
        fd[f"case{i}_ref"] = rg.SynchrotronSpectrumFromDist(dist, bins, 1.0, 1.0).as_array()
    np.savez_compressed(os.path.join(HERE, "fromdist.npz"), **fd)

    # --- distribution generators (distributions.cpp:37-136) -------------------------
    gen = {}
    bins = rg.Logbins(1e-3, 10.0, 300)
    gen["bins"] = bins.as_array()
    gen["plaw"] = rg.PlawGenerator(-1.2, 1e-2, 1.0).compute(bins).as_array()
    gen["plaw_open"] = rg.PlawGenerator(-2.5, 0.5, 0.0).compute(bins).as_array()
    gen["plaw_m1"] = rg.PlawGenerator(-1.0, 0.1, 5.0).compute(bins).as_array()
    gen["bplaw"] = rg.BrokenPlawGenerator(0.3, 0.23, -1.0, 1e-2, 2.0).compute(bins).as_array()
    gen["bplaw_open"] = rg.BrokenPlawGenerator(0.3, 0.5, -2.5, 1e-2, 0.0).compute(bins).as_array()
    gen["delta"] = rg.DeltaGenerator(2e-2, 0.01).compute(bins).as_array()
    np.savez_compressed(os.path.join(HERE, "generators.npz"), **gen)
    print("golden fixtures written to", HERE)


def make_ic(rg) -> None:
    """ICSpectrum (ic.cpp:15-46): the reference test's configuration (tests/ic.py), a
    steeper power law against a broader soft-photon field, and linear particle bins."""
    ic = {}
    cases = [("log", 1.5, 1e-8, 0.1), ("log", 2.5, 3e-9, 0.5), ("lin", 1.5, 1e-8, 0.1)]
    for i, (kind, p, e_break, width) in enumerate(cases):
        gb = rg.Logbins(1e3, 1e7, 200) if kind == "log" else rg.Linbins(1e3, 1e7, 200)
        dist_prtls = rg.TabulatedDistribution(gb, rg.PlawGenerator(-p, 1e3, 1e7))
        dist_soft = rg.TabulatedDistribution(rg.Logbins(1e-11, 1e-7, 200, rg.EnergyUnits.mec2),
                                             rg.DeltaGenerator(e_break, e_break * width))
        bins_eic = rg.Bins(rg.Logspace(1e3, 1e7, 200), rg.EnergyUnits.mec2)
        ic[f"case{i}_gb"] = dist_prtls.EnergyBins().as_array()
        ic[f"case{i}_f"] = dist_prtls.F().as_array()
        ic[f"case{i}_log"] = np.array(kind == "log")
        ic[f"case{i}_es"] = dist_soft.EnergyBins().as_array()
        ic[f"case{i}_fs"] = dist_soft.F().as_array()
        ic[f"case{i}_eic"] = bins_eic.as_array()
        ic[f"case{i}_ref"] = rg.ICSpectrum(dist_prtls, dist_soft, bins_eic).as_array()
    np.savez_compressed(os.path.join(HERE, "ic.npz"), **ic)
    print("ic.npz written to", HERE)


if __name__ == "__main__":
    if sys.argv[1:] == ["ic"]:
        make_ic(load_reference())
    else:
        main()
        make_ic(load_reference())

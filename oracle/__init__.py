"""ctypes bindings to the oracle -- TEST INFRASTRUCTURE ONLY.

The oracle (``oracle/ragnar_oracle.cpp``) restates the reference library's
synchrotron hot path on the CPU.  Only the tests, ``__graft_entry__.smoke()`` and
``bench.py`` (its ``cpu_baseline`` leg and ``--impl reference`` arm) may use this
module, and only as the checker or the CPU baseline; the product
(``ragnar_gb300``) never imports it.
"""

from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libragnar_oracle.so")

_f32p = ctypes.POINTER(ctypes.c_float)
_f64p = ctypes.POINTER(ctypes.c_double)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i64 = ctypes.c_int64
_f32 = ctypes.c_float
_int = ctypes.c_int

_lib = None


def build() -> None:
    """Compile the oracle library (make -C oracle)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


def _declare(L: ctypes.CDLL) -> None:
    P10 = [_f32p] * 10
    L.orc_linspace.argtypes = [_f32, _f32, _i64, _f32p]
    L.orc_logspace.argtypes = [_f32, _f32, _i64, _f32p]
    L.orc_ffunc_integrand.argtypes = [_f32]
    L.orc_ffunc_integrand.restype = _f32
    L.orc_tabulate_ffunc.argtypes = [_i64, _f32, _f32, _f32p, _f32p]
    L.orc_interp_log_f32.argtypes = [_f32, _f32p, _f32p, _i64, _f32, _f32, _f32]
    L.orc_interp_log_f32.restype = _f32
    L.orc_interp_log_f64.argtypes = [ctypes.c_double, _f32p, _f32p, _i64, _f32, _f32]
    L.orc_interp_log_f64.restype = ctypes.c_double
    tail = [_f32p, _i64, _f32, _f32, _f32, _f32p, _f32p, _i64]
    L.orc_sync_spectrum_ref32.argtypes = P10 + [_i64] + tail + [_f32p, _int]
    L.orc_sync_spectrum_f64.argtypes = P10 + [_i64] + tail + [_f64p, _int]
    L.orc_sync_spectrum_batched_f64.argtypes = P10 + [_i64p, _i64] + tail + [_f64p, _int]
    L.orc_energy_bin_index.argtypes = [_f32, _f32, _f32, _int, _f32, _f32, _i64]
    L.orc_energy_bin_index.restype = _i64
    L.orc_energy_bin_index_usqr.argtypes = [_f32, _int, _f32, _f32, _i64]
    L.orc_energy_bin_index_usqr.restype = _i64
    L.orc_energy_distribution.argtypes = [_f32p, _f32p, _f32p, _i64, _f32p, _i64, _int, _int,
                                          _f32p, _f64p, _i64p, _int]
    fd = [_f32p, _f32p, _i64, _i64, _int, _f32p, _i64, _f32, _f32, _f32p, _f32p, _i64]
    L.orc_sync_from_dist_ref32.argtypes = fd + [_f32p, _int]
    L.orc_sync_from_dist_f64.argtypes = fd + [_f64p, _int]
    _d = ctypes.c_double
    L.orc_smooth_coefficients.argtypes = [_i64, _d, _d, _f64p, _int]
    L.orc_exact_F.argtypes = [_d]
    L.orc_exact_F.restype = _d
    D10 = [_f64p] * 10
    sm = [_i64, _f32p, _i64, _d, _d, _d, _f32p, _i64, _d, _d]
    L.orc_sync_smooth_f64.argtypes = D10 + sm + [_f64p, _int]
    L.orc_sync_smooth_grad_f64.argtypes = D10 + sm + [_f64p, _f64p, _f64p, _f64p, _f64p, _int]
    ic = [_f32p, _f32p, _i64, _int, _f32p, _f32p, _i64, _f32p, _i64]
    L.orc_ic_spectrum_ref32.argtypes = ic + [_f32p, _int]
    L.orc_ic_spectrum_f64.argtypes = ic + [_f64p, _int]


def _p(a, ptype=_f32p):
    if a is None:
        return None
    return a.ctypes.data_as(ptype)


def _f32arr(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float32)


# ---- grids and the F table -------------------------------------------------------

def logspace(start: float, stop: float, num: int) -> np.ndarray:
    out = np.empty(num, np.float32)
    lib().orc_logspace(start, stop, num, _p(out))
    return out


def linspace(start: float, stop: float, num: int) -> np.ndarray:
    out = np.empty(num, np.float32)
    lib().orc_linspace(start, stop, num, _p(out))
    return out


def ffunc_integrand(x: float) -> float:
    return float(lib().orc_ffunc_integrand(x))


def tabulate_ffunc(n: int = 200, xmin: float = 1e-6, xmax: float = 100.0):
    xs = np.empty(n, np.float32)
    ys = np.empty(n, np.float32)
    lib().orc_tabulate_ffunc(n, xmin, xmax, _p(xs), _p(ys))
    return xs, ys


# ---- particle spectra ---------------------------------------------------------------

def _particle_args(prt: dict):
    keys = ("ux", "uy", "uz", "ex", "ey", "ez", "bx", "by", "bz", "w")
    arrs = [_f32arr(prt.get(k)) for k in keys]
    n = len(arrs[0])
    for k, a in zip(keys, arrs):
        if a is not None and len(a) != n:
            raise ValueError(f"component {k} has length {len(a)} != {n}")
    return arrs, n


def sync_spectrum_ref32(prt: dict, bins, B0, g_syn, eps, table, nthreads=0) -> np.ndarray:
    """Reference arithmetic (the port used as CPU baseline); float32 result."""
    arrs, n = _particle_args(prt)
    bins = _f32arr(bins)
    tx, ty = (_f32arr(t) for t in table)
    out = np.empty(len(bins), np.float32)
    lib().orc_sync_spectrum_ref32(*[_p(a) for a in arrs], n, _p(bins), len(bins), B0, g_syn,
                                  eps, _p(tx), _p(ty), len(tx), _p(out), nthreads)
    return out


def sync_spectrum_f64(prt: dict, bins, B0, g_syn, eps, table, nthreads=0) -> np.ndarray:
    """FP64 ground truth of the particle spectrum."""
    arrs, n = _particle_args(prt)
    bins = _f32arr(bins)
    tx, ty = (_f32arr(t) for t in table)
    out = np.empty(len(bins), np.float64)
    lib().orc_sync_spectrum_f64(*[_p(a) for a in arrs], n, _p(bins), len(bins), B0, g_syn,
                                eps, _p(tx), _p(ty), len(tx), _p(out, _f64p), nthreads)
    return out


def sync_spectrum_batched_f64(prt: dict, offsets, bins, B0, g_syn, eps, table,
                              nthreads=0) -> np.ndarray:
    arrs, n = _particle_args(prt)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    bins = _f32arr(bins)
    tx, ty = (_f32arr(t) for t in table)
    nseg = len(off) - 1
    out = np.empty((nseg, len(bins)), np.float64)
    lib().orc_sync_spectrum_batched_f64(*[_p(a) for a in arrs], _p(off, _i64p), nseg,
                                        _p(bins), len(bins), B0, g_syn, eps, _p(tx), _p(ty),
                                        len(tx), _p(out, _f64p), nthreads)
    return out


# ---- histogram ------------------------------------------------------------------------

def energy_distribution(ux, uy, uz, bins, log_spaced: bool, fourvel: bool = True, nthreads=0):
    """Returns (hist_ref32 float32, hist_f64 float64, counts int64)."""
    ux, uy, uz, bins = (_f32arr(a) for a in (ux, uy, uz, bins))
    nb = len(bins)
    h32 = np.empty(nb, np.float32)
    h64 = np.empty(nb, np.float64)
    cnt = np.empty(nb, np.int64)
    lib().orc_energy_distribution(_p(ux), _p(uy), _p(uz), len(ux), _p(bins), nb,
                                  int(log_spaced), int(fourvel), _p(h32), _p(h64, _f64p),
                                  _p(cnt, _i64p), nthreads)
    return h32, h64, cnt


def energy_bin_index(ux, uy, uz, fourvel, emin, emax, n) -> int:
    return int(lib().orc_energy_bin_index(ux, uy, uz, int(fourvel), emin, emax, n))


def energy_bin_index_usqr(usqr, fourvel, emin, emax, n) -> int:
    """Reference bin index (particles.cpp:229-243) of one float |u|^2."""
    return int(lib().orc_energy_bin_index_usqr(usqr, int(fourvel), emin, emax, n))


# ---- FromDist -----------------------------------------------------------------------

def sync_from_dist_ref32(gb, f, log_spaced, bins, g_syn, eps, table, nthreads=0):
    gb, bins = _f32arr(gb), _f32arr(bins)
    f = np.ascontiguousarray(np.atleast_2d(f), dtype=np.float32)
    tx, ty = (_f32arr(t) for t in table)
    out = np.empty((f.shape[0], len(bins)), np.float32)
    lib().orc_sync_from_dist_ref32(_p(gb), _p(f), len(gb), f.shape[0], int(log_spaced),
                                   _p(bins), len(bins), g_syn, eps, _p(tx), _p(ty), len(tx),
                                   _p(out), nthreads)
    return out


def sync_from_dist_f64(gb, f, log_spaced, bins, g_syn, eps, table, nthreads=0):
    gb, bins = _f32arr(gb), _f32arr(bins)
    f = np.ascontiguousarray(np.atleast_2d(f), dtype=np.float32)
    tx, ty = (_f32arr(t) for t in table)
    out = np.empty((f.shape[0], len(bins)), np.float64)
    lib().orc_sync_from_dist_f64(_p(gb), _p(f), len(gb), f.shape[0], int(log_spaced),
                                 _p(bins), len(bins), g_syn, eps, _p(tx), _p(ty), len(tx),
                                 _p(out, _f64p), nthreads)
    return out


# ---- differentiable (smooth) mode ---------------------------------------------------

SMOOTH_XMIN, SMOOTH_XMAX = 1e-6, 100.0


def exact_F(x: float) -> float:
    """x int_x^inf K_{5/3}, FP64 from std::cyl_bessel_k."""
    return float(lib().orc_exact_F(x))


def smooth_coefficients(nseg: int, xmin: float = SMOOTH_XMIN, xmax: float = SMOOTH_XMAX,
                        nthreads=0) -> np.ndarray:
    """Hermite segment coefficients [nseg, 4] in FP64."""
    out = np.empty((nseg, 4), np.float64)
    lib().orc_smooth_coefficients(nseg, xmin, xmax, _p(out, _f64p), nthreads)
    return out


def _f64arr(a):
    return None if a is None else np.ascontiguousarray(a, dtype=np.float64)


def _smooth_args(prt, bins, coef, xmin, xmax):
    keys = ("ux", "uy", "uz", "ex", "ey", "ez", "bx", "by", "bz", "w")
    arrs = [_f64arr(prt.get(k)) for k in keys]
    coef = np.ascontiguousarray(coef, dtype=np.float32)
    nseg = coef.shape[0]
    ln_xmin = float(np.log(xmin))
    dln = float(np.log(xmax / xmin) / nseg)
    return arrs, len(arrs[0]), _f32arr(bins), coef, nseg, ln_xmin, dln


def sync_smooth_f64(prt: dict, bins, B0, g_syn, eps, coef, xmin=SMOOTH_XMIN, xmax=SMOOTH_XMAX,
                    nthreads=0) -> np.ndarray:
    """Smooth-mode spectrum in FP64 (particle data taken as float64)."""
    arrs, n, bins, coef, nseg, lnx, dln = _smooth_args(prt, bins, coef, xmin, xmax)
    out = np.empty(len(bins), np.float64)
    lib().orc_sync_smooth_f64(*[_p(a, _f64p) for a in arrs], n, _p(bins), len(bins), B0, g_syn, eps,
                              _p(coef), nseg, lnx, dln, _p(out, _f64p), nthreads)
    return out


def sync_smooth_grad_f64(prt: dict, bins, B0, g_syn, eps, coef, gS, xmin=SMOOTH_XMIN,
                         xmax=SMOOTH_XMAX, nthreads=0):
    """(dL/dw, dL/du [3, n]) of the smooth-mode spectrum given gS = dL/dS."""
    arrs, n, bins, coef, nseg, lnx, dln = _smooth_args(prt, bins, coef, xmin, xmax)
    gS = _f64arr(gS)
    gw = np.empty(n, np.float64)
    gu = np.empty((3, n), np.float64)
    lib().orc_sync_smooth_grad_f64(*[_p(a, _f64p) for a in arrs], n, _p(bins), len(bins), B0, g_syn,
                                   eps, _p(coef), nseg, lnx, dln, _p(gS, _f64p), _p(gw, _f64p),
                                   _p(gu[0], _f64p), _p(gu[1], _f64p), _p(gu[2], _f64p), nthreads)
    return gw, gu


# ---- inverse Compton --------------------------------------------------------------------

def _ic_args(gb, fp, log_spaced, es, fs, eic):
    gb, fp, es, fs, eic = (_f32arr(a) for a in (gb, fp, es, fs, eic))
    return [_p(gb), _p(fp), len(gb), int(log_spaced), _p(es), _p(fs), len(es), _p(eic), len(eic)], len(eic), \
        (gb, fp, es, fs, eic)


def ic_spectrum_ref32(gb, fp, log_spaced, es, fs, eic, nthreads=0) -> np.ndarray:
    """ICSpectrum (ic.cpp:15-46) with the reference's float arithmetic and reduction order."""
    args, ne, keep = _ic_args(gb, fp, log_spaced, es, fs, eic)
    out = np.empty(ne, np.float32)
    lib().orc_ic_spectrum_ref32(*args, _p(out), nthreads)
    return out


def ic_spectrum_f64(gb, fp, log_spaced, es, fs, eic, nthreads=0) -> np.ndarray:
    """FP64 ground truth of the IC spectrum E^2 dN/dE."""
    args, ne, keep = _ic_args(gb, fp, log_spaced, es, fs, eic)
    out = np.empty(ne, np.float64)
    lib().orc_ic_spectrum_f64(*args, _p(out, _f64p), nthreads)
    return out

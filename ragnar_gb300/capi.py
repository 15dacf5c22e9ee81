"""ctypes binding of the C ABI (``include/ragnar_gb300.h``).

Used by the torch extension, the tests and the benchmark to call the library
exactly as a foreign caller would: plain pointers, sizes and a stream handle.
Device buffers can be anything exposing a device address (torch tensors via
``data_ptr()``).
"""

from __future__ import annotations

import ctypes
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "libragnar_gb300.so")
HEADER = os.path.join(os.path.dirname(_HERE), "include", "ragnar_gb300.h")

RG_OK = 0
RG_ALGO_AUTO, RG_ALGO_DIRECT, RG_ALGO_MOMENTS = 0, 1, 2
RG_ERR_ARGUMENT = 1
RG_ERR_CUDA = 2
RG_ERR_TIMEOUT = 3
RG_ERR_UNSUPPORTED = 4
RG_ERR_RANGE = 5
RG_TABLE_REFERENCE = 0
RG_TABLE_SMOOTH = 1

_vp = ctypes.c_void_p
_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_f32 = ctypes.c_float
_int = ctypes.c_int
_f32p = ctypes.POINTER(ctypes.c_float)


class RgError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"[status {status}] {message}")
        self.status = status


class Particles(ctypes.Structure):
    """rg_particles: device SoA pointers (0 = null)."""

    _fields_ = [("u", _vp * 3), ("e", _vp * 3), ("b", _vp * 3), ("w", _vp), ("n", _i64)]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} not built; run `python -m ragnar_gb300.build`")
        L = ctypes.CDLL(LIB_PATH)
        _declare(L)
        _lib = L
    return _lib


def _declare(L: ctypes.CDLL) -> None:
    sig = {
        "rg_init": [_int],
        "rg_finalize": [],
        "rg_device_sm_count": [ctypes.POINTER(_int)],
        "rg_malloc": [ctypes.POINTER(_vp), ctypes.c_size_t],
        "rg_free": [_vp],
        "rg_memcpy_htod": [_vp, _vp, ctypes.c_size_t, _vp],
        "rg_memcpy_dtoh": [_vp, _vp, ctypes.c_size_t, _vp],
        "rg_memcpy_dtod": [_vp, _vp, ctypes.c_size_t, _vp],
        "rg_memset": [_vp, _int, ctypes.c_size_t, _vp],
        "rg_stream_synchronize": [_vp],
        "rg_logspace": [_f32, _f32, _i64, _vp],
        "rg_linspace": [_f32, _f32, _i64, _vp],
        "rg_ffunc_integrand": [_vp, _i64, _vp, _vp],
        "rg_ffunc_table": [_i64, _f32, _f32, _vp, _vp, _vp],
        "rg_spectrum_plan_create": [_vp, _i32, _f32, _f32, _f32, _i32, ctypes.POINTER(_vp)],
        "rg_spectrum_plan_destroy": [_vp],
        "rg_spectrum_plan_reserve": [_vp, _i32],
        "rg_spectrum_plan_check": [_vp, _vp],
        "rg_spectrum_plan_probe_stage_timeout": [_vp, ctypes.c_uint32, _vp],
        "rg_spectrum_run": [_vp, ctypes.POINTER(Particles), _vp, _vp],
        "rg_spectrum_run_batched": [_vp, ctypes.POINTER(Particles), _vp, _i32, _vp, _vp],
        "rg_spectrum_run_plain": [_vp, ctypes.POINTER(Particles), _vp, _vp],
        "rg_spectrum_run_host": [_vp, ctypes.POINTER(Particles), _vp, _vp],
        "rg_spectrum_run_placed": [_vp, ctypes.POINTER(Particles), _vp, _vp, _vp],
        "rg_spectrum_adjoint_placed": [_vp, ctypes.POINTER(Particles), _vp, _vp, _vp, _vp, _vp, _vp, _vp],
        "rg_spectrum_plan_enable_timing": [_vp, _i32],
        "rg_spectrum_plan_set_algorithm": [_vp, _i32],
        "rg_spectrum_plan_algorithm": [_vp, _i32, ctypes.POINTER(_i32)],
        "rg_spectrum_plan_smooth_table": [_vp, _vp, ctypes.POINTER(_i32), ctypes.POINTER(ctypes.c_double),
                                          ctypes.POINTER(ctypes.c_double)],
        "rg_spectrum_plan_kernel_time": [_vp, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(_i64)],
        "rg_synchrotron_spectrum": [ctypes.POINTER(Particles), _vp, _i32, _f32, _f32, _f32, _vp, _vp],
        "rg_synchrotron_spectrum_noalloc": [ctypes.POINTER(Particles), _vp, _i32, _f32, _f32, _f32, _vp,
                                            _vp],
        "rg_synchrotron_spectrum_from_dist": [_vp, _vp, _i32, _i32, _vp, _i32, _f32, _f32, _vp, _vp],
        "rg_spectrum_adjoint": [_vp, ctypes.POINTER(Particles), _vp, _vp, _vp, _vp, _vp, _vp],
        "rg_spectrum_adjoint_batched": [_vp, ctypes.POINTER(Particles), _vp, _i32, _vp, _vp, _vp, _vp,
                                        _vp, _vp],
        "rg_dist_plan_create": [_vp, _i32, _f32, _f32, _i32, _i32, ctypes.POINTER(_vp)],
        "rg_dist_run": [_vp, _vp, _vp, _i32, _vp, _vp],
        "rg_dist_adjoint": [_vp, _vp, _vp, _i32, _vp, _vp, _vp],
        "rg_fromdist_plan_create": [_vp, _i32, _i32, _vp, _i32, _f32, _f32, _i32, _i32, _i32,
                                    ctypes.POINTER(_vp)],
        "rg_fromdist_plan_destroy": [_vp],
        "rg_fromdist_run": [_vp, _vp, _i32, _vp, _vp],
        "rg_fromdist_adjoint": [_vp, _vp, _i32, _vp, _vp],
        "rg_fromdist_plan_check": [_vp, _vp],
        "rg_fromdist_kernel_matrix": [_vp, _vp],
        "rg_fromdist_plan_config": [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i32), ctypes.POINTER(_i32),
                                    ctypes.POINTER(_i32)],
        "rg_fromdist_plan_set_config": [_vp, _i32, _i32],
        "rg_fromdist_plan_split_k": [_vp, ctypes.POINTER(_i32), ctypes.POINTER(_i32)],
        "rg_fromdist_plan_set_split_k": [_vp, _i32, _i32],
        "rg_ic_spectrum": [_vp, _vp, _i32, _i32, _vp, _vp, _i32, _vp, _i32, _vp, _vp],
        "rg_energy_thresholds": [_vp, _i32, _i32, _vp, ctypes.POINTER(_i32)],
        "rg_smooth_table": [_vp, ctypes.POINTER(_i32), ctypes.POINTER(ctypes.c_double),
                            ctypes.POINTER(ctypes.c_double)],
        "rg_energy_distribution": [_vp, _vp, _vp, _i64, _vp, _i32, _i32, _i32, _vp, _vp, _vp],
    }
    for name, args in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = _int
    L.rg_last_error.argtypes = []
    L.rg_last_error.restype = ctypes.c_char_p
    for name in ("rg_debug_bessel_k53", "rg_debug_exact_F"):
        fn = getattr(L, name)
        fn.argtypes = [ctypes.c_double]
        fn.restype = ctypes.c_double


def check(status: int) -> None:
    if status != RG_OK:
        msg = lib().rg_last_error().decode(errors="replace")
        raise RgError(status, msg)


def header_functions(path: str = HEADER) -> list[str]:
    """Names of every function the C ABI header declares."""
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b(rg_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def addr(t) -> int:
    """Device address of a tensor-like (0 for None)."""
    if t is None:
        return 0
    if isinstance(t, int):
        return t
    return int(t.data_ptr())


def particles(u, b=None, e=None, w=None, n=None) -> Particles:
    """Build an rg_particles from 3-sequences of device tensors (or None).  The returned
    structure holds references to the tensors, so that temporaries passed here stay
    allocated while the structure is in use."""
    p = Particles()
    p._refs = (u, b, e, w)
    for d in range(3):
        p.u[d] = addr(u[d])
        p.e[d] = addr(e[d]) if e is not None else 0
        p.b[d] = addr(b[d]) if b is not None else 0
    p.w = addr(w)
    p.n = int(n if n is not None else u[0].numel())
    return p


def host_particles(u, b=None, e=None, w=None, n=None) -> Particles:
    """rg_particles over HOST arrays (numpy arrays or pinned CPU tensors); holds references
    to the arrays like particles()."""

    def hp(a):
        if a is None:
            return 0
        if hasattr(a, "data_ptr"):
            return int(a.data_ptr())
        return int(a.ctypes.data)

    p = Particles()
    p._refs = (u, b, e, w)
    for d in range(3):
        p.u[d] = hp(u[d])
        p.e[d] = hp(e[d]) if e is not None else 0
        p.b[d] = hp(b[d]) if b is not None else 0
    p.w = hp(w)
    p.n = int(n if n is not None else len(u[0]))
    return p


class SpectrumPlan:
    """Owning wrapper of rg_spectrum_plan."""

    def __init__(self, bins, B0: float, g_syn: float, eps: float, mode: int = RG_TABLE_REFERENCE):
        import numpy as np  # noqa: PLC0415

        self.bins = np.ascontiguousarray(bins, dtype=np.float32)
        self.nbins = len(self.bins)
        h = _vp()
        check(lib().rg_spectrum_plan_create(self.bins.ctypes.data, self.nbins, B0, g_syn, eps, mode,
                                            ctypes.byref(h)))
        self.handle = h
        self.mode = mode

    def run(self, prt: Particles, out, stream: int = 0) -> None:
        check(lib().rg_spectrum_run(self.handle, ctypes.byref(prt), addr(out), stream))

    def run_plain(self, prt: Particles, out, stream: int = 0) -> None:
        check(lib().rg_spectrum_run_plain(self.handle, ctypes.byref(prt), addr(out), stream))

    def run_batched(self, prt: Particles, offsets, nseg: int, out, stream: int = 0) -> None:
        check(lib().rg_spectrum_run_batched(self.handle, ctypes.byref(prt), addr(offsets), nseg,
                                            addr(out), stream))

    def run_host(self, prt: Particles, out, stream: int = 0) -> None:
        """prt holds HOST pointers (see host_particles)."""
        check(lib().rg_spectrum_run_host(self.handle, ctypes.byref(prt), addr(out), stream))

    def enable_timing(self, on: bool = True) -> None:
        check(lib().rg_spectrum_plan_enable_timing(self.handle, int(on)))

    def set_algorithm(self, algo: int) -> None:
        """RG_ALGO_AUTO, RG_ALGO_DIRECT (the fused per-eval kernel) or RG_ALGO_MOMENTS."""
        check(lib().rg_spectrum_plan_set_algorithm(self.handle, algo))

    def smooth_table(self):
        """(coef [nseg, 4] float32, ln_xmin, dln) of the smooth table this plan evaluates."""
        import numpy as np  # noqa: PLC0415

        nseg = _i32()
        lnx, dln = ctypes.c_double(), ctypes.c_double()
        check(lib().rg_spectrum_plan_smooth_table(self.handle, None, ctypes.byref(nseg), ctypes.byref(lnx),
                                                  ctypes.byref(dln)))
        coef = np.empty((nseg.value, 4), np.float32)
        check(lib().rg_spectrum_plan_smooth_table(self.handle, coef.ctypes.data, None, None, None))
        return coef, lnx.value, dln.value

    def algorithm(self, nseg: int = 1) -> int:
        """The algorithm a run over nseg segments would use."""
        a = _i32()
        check(lib().rg_spectrum_plan_algorithm(self.handle, nseg, ctypes.byref(a)))
        return a.value

    def kernel_time(self) -> tuple[float, int]:
        """(summed fused-kernel milliseconds, launches) since the last call."""
        ms = ctypes.c_double()
        n = _i64()
        check(lib().rg_spectrum_plan_kernel_time(self.handle, ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def adjoint(self, prt: Particles, grad_out, grad_w=None, grad_u=(None, None, None),
                stream: int = 0) -> None:
        check(lib().rg_spectrum_adjoint(self.handle, ctypes.byref(prt), addr(grad_out), addr(grad_w),
                                        addr(grad_u[0]), addr(grad_u[1]), addr(grad_u[2]), stream))

    def placement_supported(self) -> bool:
        """Whether run_placed / adjoint_placed apply: cell moments on the plan's bin-aligned
        smooth table for a single segment."""
        return self.mode == RG_TABLE_SMOOTH and self.algorithm(1) == RG_ALGO_MOMENTS

    def run_placed(self, prt: Particles, out, placement, stream: int = 0) -> None:
        """run() that also writes each particle's table placement (8 bytes per particle) into
        `placement` (a device buffer of at least prt.n * 8 bytes) for adjoint_placed."""
        check(lib().rg_spectrum_run_placed(self.handle, ctypes.byref(prt), addr(out), addr(placement), stream))

    def adjoint_placed(self, prt: Particles, placement, grad_out, grad_w=None, grad_u=(None, None, None),
                       stream: int = 0) -> None:
        """adjoint() from the placement a run_placed of the same particles wrote."""
        check(lib().rg_spectrum_adjoint_placed(self.handle, ctypes.byref(prt), addr(placement), addr(grad_out),
                                               addr(grad_w), addr(grad_u[0]), addr(grad_u[1]), addr(grad_u[2]),
                                               stream))

    def adjoint_batched(self, prt: Particles, offsets, nseg: int, grad_out, grad_w=None,
                        grad_u=(None, None, None), stream: int = 0) -> None:
        check(lib().rg_spectrum_adjoint_batched(self.handle, ctypes.byref(prt), addr(offsets), nseg,
                                                addr(grad_out), addr(grad_w), addr(grad_u[0]),
                                                addr(grad_u[1]), addr(grad_u[2]), stream))

    def reserve(self, nseg: int) -> None:
        check(lib().rg_spectrum_plan_reserve(self.handle, nseg))

    def check(self, stream: int = 0) -> None:
        check(lib().rg_spectrum_plan_check(self.handle, stream))

    def probe_stage_timeout(self, polls: int, stream: int = 0) -> None:
        """Records a stage-wait timeout through a bounded wait that nothing completes."""
        check(lib().rg_spectrum_plan_probe_stage_timeout(self.handle, polls, stream))

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().rg_spectrum_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):  # noqa: D105
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass


class DistPlan(SpectrumPlan):
    """rg_spectrum_plan for a tabulated distribution (rg_dist_plan_create)."""

    def __init__(self, bins, g_syn: float, eps: float, log_spaced: bool, mode: int = RG_TABLE_REFERENCE):
        import numpy as np  # noqa: PLC0415

        self.bins = np.ascontiguousarray(bins, dtype=np.float32)
        self.nbins = len(self.bins)
        h = _vp()
        check(lib().rg_dist_plan_create(self.bins.ctypes.data, self.nbins, g_syn, eps, int(log_spaced),
                                        mode, ctypes.byref(h)))
        self.handle = h

    def run_dist(self, gbeta, f, out, stream: int = 0) -> None:
        check(lib().rg_dist_run(self.handle, addr(gbeta), addr(f), int(f.numel()), addr(out), stream))

    def adjoint_dist(self, gbeta, f, grad_out, grad_f, stream: int = 0) -> None:
        check(lib().rg_dist_adjoint(self.handle, addr(gbeta), addr(f), int(f.numel()), addr(grad_out),
                                    addr(grad_f), stream))


class FromDistPlan:
    """rg_fromdist_plan: many distributions on shared gamma bins via the tensor-core GEMM."""

    def __init__(self, gbeta, log_spaced: bool, bins, g_syn: float, eps: float, max_dist: int,
                 mode: int = RG_TABLE_REFERENCE, split_products: int = 6):
        import numpy as np  # noqa: PLC0415

        self.gbeta = np.ascontiguousarray(gbeta, dtype=np.float32)
        self.bins = np.ascontiguousarray(bins, dtype=np.float32)
        self.ng, self.nbins, self.max_dist = len(self.gbeta), len(self.bins), max_dist
        h = _vp()
        check(lib().rg_fromdist_plan_create(self.gbeta.ctypes.data, self.ng, int(log_spaced),
                                            self.bins.ctypes.data, self.nbins, g_syn, eps, mode,
                                            split_products, max_dist, ctypes.byref(h)))
        self.handle = h

    def run(self, f, out, stream: int = 0) -> None:
        check(lib().rg_fromdist_run(self.handle, addr(f), int(f.shape[0]), addr(out), stream))

    def adjoint(self, grad_out, grad_f, stream: int = 0) -> None:
        check(lib().rg_fromdist_adjoint(self.handle, addr(grad_out), int(grad_out.shape[0]), addr(grad_f), stream))

    def check(self, stream: int = 0) -> None:
        check(lib().rg_fromdist_plan_check(self.handle, stream))

    def config(self) -> dict:
        """Autotuned tile shapes {"fwd": (bn, stages), "adj": (bn, stages)}."""
        v = [_i32() for _ in range(4)]
        check(lib().rg_fromdist_plan_config(self.handle, *[ctypes.byref(x) for x in v]))
        return {"fwd": (v[0].value, v[1].value), "adj": (v[2].value, v[3].value)}

    def set_config(self, fwd: int = -1, adj: int = -1) -> None:
        check(lib().rg_fromdist_plan_set_config(self.handle, fwd, adj))

    def split_k(self) -> dict:
        """Autotuned split-K range counts {"fwd": n, "adj": n} (1: no split)."""
        v = [_i32() for _ in range(2)]
        check(lib().rg_fromdist_plan_split_k(self.handle, *[ctypes.byref(x) for x in v]))
        return {"fwd": v[0].value, "adj": v[1].value}

    def set_split_k(self, fwd: int = -1, adj: int = -1) -> None:
        check(lib().rg_fromdist_plan_set_split_k(self.handle, fwd, adj))

    def kernel_matrix(self):
        import numpy as np  # noqa: PLC0415

        K = np.empty((self.nbins, self.ng), np.float64)
        check(lib().rg_fromdist_kernel_matrix(self.handle, K.ctypes.data))
        return K

    def close(self) -> None:
        if getattr(self, "handle", None):
            lib().rg_fromdist_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):  # noqa: D105
        try:
            self.close()
        except Exception:  # noqa: BLE001
            pass

"""ctypes binding of ``libgcpm.so`` (declared in ``include/gcpm.h``).

This is the only way the package reaches the device: every operator of the PM
chain is a call into the CUDA library. There is no CPU fallback; when the
library is missing or CUDA is unavailable, :func:`lib` raises.
"""

from __future__ import annotations

import ctypes as C
import threading
from pathlib import Path

from galaxy_collision_gb300._build import LIB_PATH

GC_OK = 0
GC_ERR_ARG = -1
GC_ERR_CUDA = -2
GC_ERR_TIMEOUT = -3
GC_ERR_NOT_CONVERGED = -4
GC_ERR_NONFINITE = -5
GC_ERR_STATE = -6

GC_FLAG_NONFINITE_POS = 0x1
GC_FLAG_NONFINITE_RHO = 0x2
GC_FLAG_BAD_PID = 0x4
GC_FLAG_IC_REJECT = 0x8
GC_FLAG_TIMEOUT = 0x10
GC_MG_FIXED_CYCLES = 0x2
GC_MG_PLAIN_F32 = 0x4
GC_MG_NATURAL_LAYOUT = 0x8
GC_MG_FACES_GIVEN = 0x10
GC_MG_PHASE_LAUNCHES = 0x20
GC_MG_COARSE_ONE_SWEEP = 0x40
GC_STEP_GRAD_GRID = 0x1
GC_STEP_SOLVE_ONLY = 0x2
GC_STEP_PUSH_ONLY = 0x4
GC_STEP_DEPOSIT_NEXT = 0x8

GC_WS_PLAIN = 0
GC_WS_LEARNED = 1
GC_WS_EXTRAPOLATE = 2

GC_STEP_PRIME = 0
GC_STEP_ADVANCE = 1
GC_STEP_CLOSE = 2

_fp = C.POINTER(C.c_float)
_vp = C.c_void_p
_i64 = C.c_int64
_ctxp = C.c_void_p


class MGParams(C.Structure):
    _fields_ = [
        ("pre_sweeps", C.c_int),
        ("post_sweeps", C.c_int),
        ("coarse_sweeps", C.c_int),
        ("max_cycles", C.c_int),
        ("min_cycles", C.c_int),
        ("flags", C.c_int),
        ("tol", C.c_double),
    ]


class MGStats(C.Structure):
    _fields_ = [
        ("cycles", C.c_int),
        ("converged", C.c_int),
        ("rhs_norm", C.c_double),
        ("res_norm", C.c_double),
    ]


class Particles(C.Structure):
    _fields_ = [
        ("x", _vp), ("y", _vp), ("z", _vp),
        ("vx", _vp), ("vy", _vp), ("vz", _vp),
        ("m", _vp), ("gid", _vp), ("pid", _vp),
        ("n", _i64),
    ]


class StepParams(C.Structure):
    _fields_ = [
        ("dt", C.c_float),
        ("mode", C.c_int),
        ("warm_start", C.c_int),
        ("diagnostics", C.c_int),
        ("mg", MGParams),
        ("fixed_point_bits", C.c_int),
        ("flags", C.c_int),
    ]


class StepStats(C.Structure):
    _fields_ = [
        ("mg", MGStats),
        ("diag", C.c_double * 11),
        ("grid_pe_raw", C.c_double),
    ]


# name -> (restype, argtypes)
_PROTOS = {
    "gc_abi_version": (C.c_int, []),
    "gc_last_error": (C.c_char_p, [_ctxp]),
    "gc_ctx_create": (C.c_int, [C.POINTER(_ctxp), C.c_int, C.c_double, C.c_double]),
    "gc_ctx_destroy": (C.c_int, [_ctxp]),
    "gc_set_stream": (C.c_int, [_ctxp, _vp]),
    "gc_status": (C.c_int, [_ctxp, C.POINTER(C.c_uint32), C.c_int]),
    "gc_num_levels": (C.c_int, [_ctxp]),
    "gc_level_info": (C.c_int, [_ctxp, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "gc_deposit_cic": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp, _i64, C.c_int, _vp]),
    "gc_selftest_wait_timeout": (C.c_int, [_vp, _vp, _i64, C.c_int]),
    "gc_deposit_cic_noalloc": (C.c_int, [_vp, _vp, _vp, _vp, _i64, C.c_int, C.c_double, C.c_int, _vp, _vp, _vp]),
    "gc_potential_to_accel": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp]),
    "gc_gather_accel": (C.c_int, [_ctxp, _vp, _vp, _vp, _i64, _vp, _vp, _vp, _vp, _vp, _vp]),
    "gc_kick": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, C.c_float]),
    "gc_drift": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, C.c_float]),
    "gc_cell_keys": (C.c_int, [_ctxp, _vp, _vp, _vp, _i64, _vp]),
    "gc_sort_keys": (C.c_int, [_ctxp, _vp, _i64, _vp, _vp]),
    "gc_mg_default_params": (None, [C.POINTER(MGParams)]),
    "gc_mg_solve": (C.c_int, [_ctxp, _vp, _vp, C.c_int, C.POINTER(MGParams), C.POINTER(MGStats)]),
    "gc_mg_residual_norm": (C.c_int, [_ctxp, _vp, C.POINTER(C.c_double)]),
    "gc_moments": (C.c_int, [_ctxp, _vp, C.POINTER(C.c_double)]),
    "gc_diag_particles": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i64, C.POINTER(C.c_double)]),
    "gc_diag_grid_pe": (C.c_int, [_ctxp, _vp, _vp, C.POINTER(C.c_double)]),
    "gc_radial_histogram": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp, _i64, C.c_double, C.c_double, C.c_double,
                                      C.c_double, C.c_int, _vp]),
    "gc_project_ngp": (C.c_int, [_ctxp, _vp, _vp, _vp, _i64, C.c_double, C.c_double, C.c_double, C.c_double,
                                 C.c_int, _vp]),
    "gc_rng_uniform": (C.c_int, [_ctxp, C.c_uint64, C.c_uint32, _i64, _vp]),
    "gc_ic_plummer": (C.c_int, [_ctxp, _i64, C.c_uint64, C.c_double, C.c_double, C.c_double, C.c_double, _vp, _vp,
                                _vp, _vp]),
    "gc_ic_disk": (C.c_int, [_ctxp, _i64, C.c_uint64, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double,
                             C.c_double, C.POINTER(C.c_double), C.POINTER(C.c_double), _vp, _vp, _vp, _vp]),
    "gc_max_f32": (C.c_int, [_ctxp, _vp, _i64, _vp]),
    "gc_colormap_log": (C.c_int, [_ctxp, _vp, _i64, _vp, C.c_float, C.c_float, _vp]),
    "gc_pack_positions": (C.c_int, [_ctxp, _vp, _vp, _vp, _i64, C.c_float, _i64, _vp]),
    "gc_density_color": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp, C.c_int, _i64, _i64, C.c_float, _vp, C.c_float,
                                   C.c_float, _vp]),
    "gc_splat_points": (C.c_int, [_ctxp, _vp, _vp, _i64, C.POINTER(C.c_float), C.c_int, C.c_int, C.c_float,
                                  C.POINTER(C.c_float), _vp, _vp]),
    "gc_pm_sort": (C.c_int, [_ctxp, C.POINTER(Particles), C.POINTER(Particles)]),
    "gc_pm_sort_ahead": (C.c_int, [_ctxp, C.POINTER(Particles), C.POINTER(Particles), C.c_float]),
    "gc_pm_reserve": (C.c_int, [_ctxp, _i64]),
    "gc_pm_import": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp, C.POINTER(C.c_double), C.POINTER(Particles)]),
    "gc_pm_import_sorted": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp, C.POINTER(C.c_double), C.POINTER(Particles)]),
    "gc_pm_import_order": (C.c_int, [_ctxp, _vp, C.POINTER(C.c_double), _i64]),
    "gc_pm_import_gather": (C.c_int, [_ctxp, _vp, _vp, _vp, _vp, C.POINTER(C.c_double), C.POINTER(Particles)]),
    "gc_pm_export": (C.c_int, [_ctxp, C.POINTER(Particles), C.POINTER(C.c_double), _vp, _vp, _vp, _vp]),
    "gc_pm_export_order": (C.c_int, [_ctxp, C.POINTER(Particles)]),
    "gc_pm_export_range": (C.c_int, [_ctxp, C.POINTER(Particles), C.POINTER(C.c_double), _vp, _vp, _vp, _vp, _i64,
                                     _i64]),
    "gc_pm_step": (C.c_int, [_ctxp, C.POINTER(Particles), C.POINTER(StepParams), C.POINTER(StepStats)]),
    "gc_pm_potential": (_vp, [_ctxp]),
    "gc_pm_copy_potential": (C.c_int, [_ctxp, _vp]),
    "gc_pm_last_residual": (C.c_int, [_ctxp, C.POINTER(C.c_double)]),
    "gc_pm_residual_host": (C.c_int, [_ctxp, C.POINTER(C.c_double)]),
    "gc_pm_refine": (C.c_int, [_ctxp, C.POINTER(MGParams), C.POINTER(C.c_int)]),
    "gc_profile_enable": (C.c_int, [_ctxp, C.c_int]),
    "gc_profile_reset": (C.c_int, [_ctxp]),
    "gc_profile_read": (C.c_int, [_ctxp, C.c_int, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                  C.POINTER(C.c_double)]),
    "gc_num_kernel_ids": (C.c_int, []),
    "gc_kernel_name": (C.c_char_p, [C.c_int]),
    "gc_ws_selftest_gemm": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _vp, _vp]),
    "gc_ws_create": (C.c_int, [C.POINTER(_vp), C.c_int]),
    "gc_ws_destroy": (C.c_int, [_vp]),
    "gc_ws_last_error": (C.c_char_p, [_vp]),
    "gc_ws_set_stream": (C.c_int, [_vp, _vp]),
    "gc_ws_layer_info": (C.c_int, [C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int),
                                   C.POINTER(C.c_int)]),
    "gc_ws_num_params": (C.c_int, [_vp, C.POINTER(_i64)]),
    "gc_ws_set_params": (C.c_int, [_vp, _vp]),
    "gc_ws_get_params": (C.c_int, [_vp, _vp]),
    "gc_ws_get_grads": (C.c_int, [_vp, _vp]),
    "gc_ws_forward": (C.c_int, [_vp, _vp, _vp]),
    "gc_ws_backward": (C.c_int, [_vp, _vp, _vp]),
    "gc_ws_adam": (C.c_int, [_vp, C.c_float, C.c_float, C.c_float, C.c_float, C.c_int]),
    "gc_ws_status": (C.c_int, [_vp, C.POINTER(C.c_uint32), C.c_int]),
    "gc_ws_autotune": (C.c_int, [_vp, C.c_int, _vp]),
    "gc_ws_plan_info": (C.c_int, [_vp, C.c_int, C.c_int, _vp]),
    "gc_pm_graph_create": (C.c_int, [_ctxp, C.POINTER(Particles), C.POINTER(StepParams), C.POINTER(_vp)]),
    "gc_pm_graph_launch": (C.c_int, [_vp]),
    "gc_pm_graph_destroy": (C.c_int, [_vp]),
    "gc_pm_graph_info": (C.c_int, [_vp, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "gc_pm_graph_stats": (C.c_int, [_ctxp, C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_double)]),
    "gc_pm_solve_counters": (C.c_int, [_ctxp, C.POINTER(C.c_double), C.c_int]),
    "gc_pm_set_warmstart": (C.c_int, [_ctxp, _vp, C.c_int, C.c_int]),
    "gc_pm_record_sample": (C.c_int, [_ctxp, _vp]),
}

EXPORTED = tuple(_PROTOS)

_lock = threading.Lock()
_lib = None


def library_path() -> Path:
    return LIB_PATH


def load(path: Path | None = None) -> C.CDLL:
    """Load the shared library without touching the GPU (no CUDA call is made)."""
    global _lib
    with _lock:
        if _lib is not None and path is None:
            return _lib
        p = Path(path) if path else LIB_PATH
        if not p.exists():
            raise RuntimeError(
                f"libgcpm.so not found at {p}; build it with galaxy_collision_gb300._build.build() "
                "(the CUDA library is required, there is no CPU fallback)"
            )
        lib = C.CDLL(str(p))
        for name, (res, args) in _PROTOS.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        if lib.gc_abi_version() != 1:
            raise RuntimeError("libgcpm.so ABI version mismatch")
        if path is None:
            _lib = lib
        return lib


def lib() -> C.CDLL:
    """The loaded library, requiring a CUDA device (raises otherwise)."""
    import torch

    if not torch.cuda.is_available():
        raise RuntimeError("galaxy_collision_gb300 needs a CUDA device: the PM chain runs only on the GPU")
    return load()


class GCError(RuntimeError):
    pass


def check(status: int, ctx=None, what: str = "") -> None:
    if status == GC_OK:
        return
    msg = load().gc_last_error(ctx)
    msg = msg.decode() if msg else ""
    text = f"{what}: {msg}" if what else msg
    if status == GC_ERR_ARG:
        raise ValueError(text)
    raise GCError(f"[status {status}] {text}")


def ptr(t) -> int:
    """Raw device pointer of a CUDA tensor (or 0 for None)."""
    if t is None:
        return None
    return t.data_ptr()


def current_stream_handle():
    import torch

    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class Context:
    """Owns one ``gc_ctx`` (grid hierarchy, int64 mass grid, scratch) on the current device."""

    def __init__(self, grid_size: int, dx: float, grav: float):
        L = lib()
        h = _ctxp()
        st = L.gc_ctx_create(C.byref(h), int(grid_size), float(dx), float(grav))
        if st != GC_OK:
            msg = L.gc_last_error(None)
            msg = msg.decode() if msg else ""
            if st == GC_ERR_ARG:
                raise ValueError(msg)
            raise GCError(msg)
        self._h = h
        self._lib = L
        self.grid_size = int(grid_size)
        self.dx = float(dx)
        self.grav = float(grav)

    @property
    def handle(self):
        return self._h

    def bind_stream(self) -> None:
        self._lib.gc_set_stream(self._h, current_stream_handle())

    def call(self, name: str, *args, what: str | None = None):
        self.bind_stream()
        st = getattr(self._lib, name)(self._h, *args)
        check(st, self._h, what or name)
        return st

    def levels(self):
        out = []
        for lv in range(self._lib.gc_num_levels(self._h)):
            n, J, p = C.c_int(), C.c_int(), C.c_double()
            self._lib.gc_level_info(self._h, lv, C.byref(n), C.byref(J), C.byref(p))
            out.append((n.value, J.value, p.value))
        return out

    def status(self, clear: bool = False) -> int:
        self.bind_stream()
        f = C.c_uint32()
        check(self._lib.gc_status(self._h, C.byref(f), int(clear)), self._h, "gc_status")
        return int(f.value)

    def profile(self, enable: bool = True) -> None:
        check(self._lib.gc_profile_enable(self._h, int(enable)), self._h, "profile")

    def profile_reset(self) -> None:
        self.bind_stream()
        check(self._lib.gc_profile_reset(self._h), self._h, "profile reset")

    def kernel_stats(self) -> dict:
        """{kernel name: (launches, timed launches, total ms)} since the last reset."""
        self.bind_stream()
        out = {}
        for kid in range(self._lib.gc_num_kernel_ids()):
            n, t, ms = C.c_longlong(), C.c_longlong(), C.c_double()
            check(self._lib.gc_profile_read(self._h, kid, C.byref(n), C.byref(t), C.byref(ms)), self._h, "profile")
            name = self._lib.gc_kernel_name(kid).decode()
            if n.value:
                out[name] = (int(n.value), int(t.value), float(ms.value))
        return out

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._lib.gc_ctx_destroy(self._h)
            self._h = _ctxp()

    def __del__(self):  # pragma: no cover - interpreter shutdown ordering
        try:
            self.close()
        except Exception:
            pass


class StepGraph:
    """One captured ADVANCE step (``gc_pm_graph_create``): replay it with
    :meth:`launch` on the stream it was captured on."""

    def __init__(self, ctx: Context, particles: Particles, params: StepParams):
        h = _vp()
        ctx.call("gc_pm_graph_create", C.byref(particles), C.byref(params), C.byref(h), what="gc_pm_graph_create")
        self._h = h
        self._ctx = ctx
        fixed, body = C.c_longlong(), C.c_longlong()
        check(ctx._lib.gc_pm_graph_info(h, C.byref(fixed), C.byref(body)), ctx.handle, "gc_pm_graph_info")
        self.fixed_launches = int(fixed.value)
        self.body_launches = int(body.value)

    def launch(self) -> None:
        check(self._ctx._lib.gc_pm_graph_launch(self._h), self._ctx.handle, "gc_pm_graph_launch")

    def close(self) -> None:
        if getattr(self, "_h", None) is not None and self._h.value:
            self._ctx._lib.gc_pm_graph_destroy(self._h)
            self._h = _vp()

    def __del__(self):  # pragma: no cover - interpreter shutdown ordering
        try:
            self.close()
        except Exception:
            pass


def default_mg_params() -> MGParams:
    p = MGParams()
    load().gc_mg_default_params(C.byref(p))
    return p

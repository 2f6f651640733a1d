"""ctypes wrapper of the C oracle (test infrastructure only; see oracle/__init__.py)."""

from __future__ import annotations

import ctypes as C

import numpy as np

from oracle.build import build

_lib = None
_f = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_d = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_u32 = np.ctypeslib.ndpointer(dtype=np.uint32, flags="C_CONTIGUOUS")
_i64 = np.ctypeslib.ndpointer(dtype=np.int64, flags="C_CONTIGUOUS")


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(str(build()))
        L.or_num_threads.restype = C.c_int
        L.or_set_threads.argtypes = [C.c_int]
        L.or_cell_keys.argtypes = [_f, _f, _f, C.c_int64, C.c_float, C.c_int, _u32]
        L.or_deposit_f32.argtypes = [_f, _f, _f, _f, C.c_int64, C.c_float, C.c_int, _f, C.c_int]
        L.or_deposit_f64.argtypes = [_f, _f, _f, _f, C.c_int64, C.c_float, C.c_int, _d]
        L.or_deposit_fixed.argtypes = [_f, _f, _f, _f, C.c_int64, C.c_float, C.c_int, C.c_int, _f, _i64]
        L.or_deposit_fixed.restype = C.c_int
        L.or_grad.argtypes = [_f, C.c_int, C.c_float, _f, _f, _f]
        L.or_gather.argtypes = [_f, _f, _f, C.c_int64, _f, _f, _f, C.c_float, C.c_int, _f, _f, _f]
        L.or_axpy3.argtypes = [_f, _f, _f, _f, _f, _f, C.c_int64, C.c_float]
        L.or_mg_create.restype = C.c_void_p
        L.or_mg_create.argtypes = [C.c_int, C.c_float, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                   C.c_int]
        L.or_mg_destroy.argtypes = [C.c_void_p]
        L.or_mg_levels.argtypes = [C.c_void_p, np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")]
        L.or_mg_levels.restype = C.c_int
        L.or_mg_vcycle.argtypes = [C.c_void_p]
        L.or_mg_solve.argtypes = [C.c_void_p, _f, _f, C.c_int, _d]
        L.or_mg_solve.restype = C.c_int
        L.or_mg_residual_norm.argtypes = [C.c_void_p]
        L.or_mg_residual_norm.restype = C.c_double
        L.or_moments.argtypes = [_f, C.c_int, C.c_float, _d]
        L.or_residual64.argtypes = [_f, _d, C.c_int, C.c_float, C.c_double, C.POINTER(C.c_double)]
        L.or_residual64.restype = C.c_double
        L.or_mg64_create.restype = C.c_void_p
        L.or_mg64_create.argtypes = [C.c_int, C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                     C.c_int]
        L.or_mg64_destroy.argtypes = [C.c_void_p]
        L.or_mg64_solve.argtypes = [C.c_void_p, _f, _d, C.c_int, _d]
        L.or_mg64_solve.restype = C.c_int
        _lib = L
    return _lib


def _f32(a):
    return np.ascontiguousarray(a, dtype=np.float32)


def num_threads() -> int:
    return lib().or_num_threads()


def set_threads(n: int) -> None:
    lib().or_set_threads(int(n))


def cell_keys(pos, dx, G):
    pos = np.asarray(pos)
    n = pos.shape[0]
    keys = np.empty(n, np.uint32)
    lib().or_cell_keys(_f32(pos[:, 0]), _f32(pos[:, 1]), _f32(pos[:, 2]), n, float(dx), int(G), keys)
    return keys


def stable_sort_perm(keys):
    """The unique stable-sort permutation (sorted position -> original index)."""
    return np.argsort(np.asarray(keys), kind="stable").astype(np.uint32)


def deposit_f32(pos, mass, dx, G, parallel=False):
    pos = np.asarray(pos)
    rho = np.zeros((G, G, G), np.float32)
    lib().or_deposit_f32(_f32(pos[:, 0]), _f32(pos[:, 1]), _f32(pos[:, 2]), _f32(mass), pos.shape[0], float(dx),
                         int(G), rho, int(parallel))
    return rho


def deposit_f64(pos, mass, dx, G):
    pos = np.asarray(pos)
    rho = np.zeros((G, G, G), np.float64)
    lib().or_deposit_f64(_f32(pos[:, 0]), _f32(pos[:, 1]), _f32(pos[:, 2]), _f32(mass), pos.shape[0], float(dx),
                         int(G), rho)
    return rho


def deposit_fixed(pos, mass, dx, G, bits=52):
    pos = np.asarray(pos)
    rho = np.zeros((G, G, G), np.float32)
    q = np.zeros((G, G, G), np.int64)
    E = lib().or_deposit_fixed(_f32(pos[:, 0]), _f32(pos[:, 1]), _f32(pos[:, 2]), _f32(mass), pos.shape[0],
                               float(dx), int(G), int(bits), rho, q)
    return rho, q, E


def grad(phi, dx):
    phi = _f32(phi)
    G = phi.shape[0]
    ax, ay, az = (np.zeros_like(phi) for _ in range(3))
    lib().or_grad(phi, G, float(dx), ax, ay, az)
    return ax, ay, az


def gather(pos, axg, ayg, azg, dx):
    pos = np.asarray(pos)
    n = pos.shape[0]
    G = axg.shape[0]
    out = [np.zeros(n, np.float32) for _ in range(3)]
    lib().or_gather(_f32(pos[:, 0]), _f32(pos[:, 1]), _f32(pos[:, 2]), n, _f32(axg), _f32(ayg), _f32(azg),
                    float(dx), G, *out)
    return out


def axpy3(u, v, w, a, b, c, dt):
    """In place: u += a*dt etc. (kick with (v, a) or drift with (x, v)); arrays must be f32 contiguous."""
    lib().or_axpy3(u, v, w, _f32(a), _f32(b), _f32(c), u.shape[0], float(dt))


def moments(rho, dx):
    out = np.zeros(10, np.float64)
    rho = _f32(rho)
    lib().or_moments(rho, rho.shape[0], float(dx), out)
    return out


def residual64(rho, phi64, dx, grav):
    rho = _f32(rho)
    bn = C.c_double()
    rn = lib().or_residual64(rho, np.ascontiguousarray(phi64, dtype=np.float64), rho.shape[0], float(dx),
                             float(grav), C.byref(bn))
    return rn, bn.value


class ReferenceMultigrid:
    """The reference MultigridPoissonSolver (solver/multigrid.py:298-494) restated in C."""

    def __init__(self, grid_size, dx=1.0, grav_constant=1.0, n_cycles=20, pre_sweeps=2, post_sweeps=2,
                 coarse_sweeps=40, tol=1e-3, min_cycles=1):
        self.grid_size = int(grid_size)
        self.dx = float(dx)
        self.G = float(grav_constant)
        self._h = lib().or_mg_create(self.grid_size, self.dx, self.G, int(n_cycles), int(pre_sweeps),
                                     int(post_sweeps), int(coarse_sweeps), float(tol), int(min_cycles))
        self.last_cycles = 0
        self.norms = np.zeros(2)

    @property
    def sizes(self):
        s = np.zeros(32, np.int32)
        n = lib().or_mg_levels(self._h, s)
        return [int(v) for v in s[:n]]

    def solve(self, rho, phi, warm_start=False):
        """rho: (G,G,G) array; phi: f32 C-contiguous array updated in place."""
        self.last_cycles = lib().or_mg_solve(self._h, _f32(rho), phi, int(bool(warm_start)), self.norms)

    def vcycle(self):
        lib().or_mg_vcycle(self._h)

    def residual_norm(self):
        return lib().or_mg_residual_norm(self._h)

    def __del__(self):
        try:
            lib().or_mg_destroy(self._h)
        except Exception:
            pass


class ReferenceMultigrid64:
    """The reference multigrid (solver/multigrid.py:298-494) in FP64 throughout:
    the same algorithm driven below the FP32 floor (the CPU baseline at 1e-6)."""

    def __init__(self, grid_size, dx=1.0, grav_constant=1.0, n_cycles=100, pre_sweeps=2, post_sweeps=2,
                 coarse_sweeps=40, tol=1e-6, min_cycles=1):
        self.grid_size = int(grid_size)
        self._h = lib().or_mg64_create(self.grid_size, float(dx), float(grav_constant), int(n_cycles),
                                       int(pre_sweeps), int(post_sweeps), int(coarse_sweeps), float(tol),
                                       int(min_cycles))
        self.last_cycles = 0
        self.norms = np.zeros(2)

    def solve(self, rho, phi64, warm_start=False):
        """rho: (G,G,G); phi64: float64 C-contiguous array updated in place."""
        self.last_cycles = lib().or_mg64_solve(self._h, _f32(rho), phi64, int(bool(warm_start)), self.norms)

    def __del__(self):
        try:
            lib().or_mg64_destroy(self._h)
        except Exception:
            pass

"""Open-boundary multigrid Poisson solver on the GPU.

Drop-in for ``MultigridPoissonSolver`` (src/galaxy_collision/solver/multigrid.py:298-494):
same constructor keywords, the same adaptive stopping rule (stop once
||rhs - L phi||_2 < tol * ||rhs||_2, never before ``min_cycles``, at most
``n_cycles``), ``last_cycles`` and ``residual_norm()``. The discrete problem is
the reference's: 7-point Laplacian on the finest grid, Dirichlet faces from the
monopole + quadrupole of rho about its centre of mass. What differs is how it
is solved (see ``csrc/multigrid.cu``): Shortley-Weller coarse levels that
converge at ~0.1 per V-cycle instead of the reference's ~0.6, a double-float
finest level so the residual can go below the FP32 floor, device-side moments
and norms, and an FP64 coarsest solve.

``boundary="isolated"`` (an addition) replaces the multipole faces by the exact
free-space boundary values of the discrete problem, by James's method: solve
with zero faces (phi0), take the screening charge phi0 leaves on the boundary
nodes (the 7-point Laplacian of phi0 continued by zero there: the sum of its
interior neighbours), evaluate its potential and that of rho's own boundary
nodes on the faces with the lattice Green's function of the 7-point stencil
(the FP64 zero-padded FFT convolution of ``FFTPoissonSolver(green="lattice")``),
and solve again with those faces. The result is the free-space solution of the
7-point problem (the lattice-Green potential) up to the solver tolerance.
"""

from __future__ import annotations

import ctypes as C

from galaxy_collision_gb300 import _native, units
from galaxy_collision_gb300.data import as_tensor
from galaxy_collision_gb300.solver.base import PoissonSolver


class MultigridPoissonSolver(PoissonSolver):
    """Open-BC Poisson solve by red-black Gauss-Seidel multigrid V-cycles (sm_103a)."""

    def __init__(
        self,
        grid_size: int,
        dx: float = 1.0,
        grav_constant: float | None = None,
        n_cycles: int = 20,
        pre_sweeps: int = 2,
        post_sweeps: int = 2,
        coarse_sweeps: int = 40,
        tol: float = 1e-3,
        min_cycles: int = 1,
        *,
        plain_f32: bool = False,
        natural_layout: bool = False,
        boundary: str = "multipole",
        phase_launches: bool = False,
        coarse_level_sweeps: int | None = None,
    ):
        self.grid_size = int(grid_size)
        self.dx = float(dx)
        self.G = units.G if grav_constant is None else float(grav_constant)
        self.n_cycles = int(n_cycles)
        self.nu1 = int(pre_sweeps)
        self.nu2 = int(post_sweeps)
        self.coarse_sweeps = int(coarse_sweeps)
        self.tol = float(tol)
        self.min_cycles = max(1, int(min_cycles))
        self.last_cycles = 0
        self.last_stats = None
        # plain_f32: the all-FP32 method (potential, residual and corrections in
        # f32; stalls at the FP32 floor like the reference), the baseline the
        # mixed-precision default is compared with
        self.plain_f32 = bool(plain_f32)
        # natural_layout: validation path, the finest correction in natural
        # layout through the generic level kernels (identical potentials)
        self.natural_layout = bool(natural_layout)
        # phase_launches: the coarse levels by one launch per phase instead of
        # the persistent kernels (identical potentials)
        self.phase_launches = bool(phase_launches)
        # coarse_level_sweeps=1: one sweep each way below the finest level (the
        # engine's default); None keeps pre/post sweeps on every level, as the reference
        if coarse_level_sweeps not in (None, 1):
            raise ValueError("coarse_level_sweeps must be None or 1")
        self.coarse_one_sweep = coarse_level_sweeps == 1
        if boundary not in ("multipole", "isolated"):
            raise ValueError(f"unknown boundary {boundary!r} (expected 'multipole' or 'isolated')")
        self.boundary = boundary
        self._lattice = None
        self._ctx = _native.Context(self.grid_size, self.dx, self.G)
        self.sizes = [n for (n, _J, _p) in self._ctx.levels()]

    def _params(self) -> _native.MGParams:
        p = _native.MGParams()
        p.pre_sweeps = self.nu1
        p.post_sweeps = self.nu2
        p.coarse_sweeps = self.coarse_sweeps
        p.max_cycles = self.n_cycles
        p.min_cycles = self.min_cycles
        p.tol = self.tol
        p.flags = ((_native.GC_MG_PLAIN_F32 if self.plain_f32 else 0)
                   | (_native.GC_MG_NATURAL_LAYOUT if self.natural_layout else 0)
                   | (_native.GC_MG_PHASE_LAUNCHES if self.phase_launches else 0)
                   | (_native.GC_MG_COARSE_ONE_SWEEP if self.coarse_one_sweep else 0))
        return p

    def solve(self, rho, phi, warm_start: bool = False) -> None:
        G = self.grid_size
        r = as_tensor(rho, shape=(G, G, G), name="rho")
        f = as_tensor(phi, shape=(G, G, G), name="phi")
        if self.boundary == "isolated":
            self._solve_isolated(r, f)
            return
        self._solve(r, f, warm_start, self._params())

    def isolated_faces(self, rho, phi0):
        """The free-space potential of rho on the boundary nodes (FP64, G^3 with
        the interior zero), from phi0, the solution with zero faces."""
        import torch

        from galaxy_collision_gb300.solver.fft import FFTPoissonSolver

        G = self.grid_size
        if self._lattice is None:
            self._lattice = FFTPoissonSolver(G, dx=self.dx, grav_constant=self.G, green="lattice")
        p0 = phi0.to(torch.float64)
        # screening charge: L phi0 on the boundary nodes, phi0 continued by zero
        s = torch.zeros_like(p0)
        s[0, 1:-1, 1:-1] = p0[1, 1:-1, 1:-1]
        s[-1, 1:-1, 1:-1] = p0[-2, 1:-1, 1:-1]
        s[1:-1, 0, 1:-1] = p0[1:-1, 1, 1:-1]
        s[1:-1, -1, 1:-1] = p0[1:-1, -2, 1:-1]
        s[1:-1, 1:-1, 0] = p0[1:-1, 1:-1, 1]
        s[1:-1, 1:-1, -1] = p0[1:-1, 1:-1, -2]
        # phi_free = phi0 + g * s on Z^3 (L g = -delta); FFTPoissonSolver(lattice)
        # returns -4 pi G dx^2 (g * src), so s enters as -s / (4 pi G dx^2); the
        # boundary nodes' own mass (which the interior equations never see) as is
        src = -s / (4.0 * 3.141592653589793 * self.G * self.dx**2)
        rb = rho.to(torch.float64)
        src[0] += rb[0]
        src[-1] += rb[-1]
        src[1:-1, 0] += rb[1:-1, 0]
        src[1:-1, -1] += rb[1:-1, -1]
        src[1:-1, 1:-1, 0] += rb[1:-1, 1:-1, 0]
        src[1:-1, 1:-1, -1] += rb[1:-1, 1:-1, -1]
        faces = self._lattice.potential64(src)
        faces[1:-1, 1:-1, 1:-1] = 0.0
        return faces

    def _solve_isolated(self, r, f) -> None:
        p = self._params()
        p.flags |= _native.GC_MG_FACES_GIVEN
        f.zero_()
        self._solve(r, f, False, p)  # phi0: zero faces
        cycles0 = self.last_cycles
        faces = self.isolated_faces(r, f)
        interior = f[1:-1, 1:-1, 1:-1].clone()
        f.copy_(faces.to(f.dtype))
        f[1:-1, 1:-1, 1:-1] = interior  # phi0 as the initial guess
        self._solve(r, f, True, p)
        self.last_stats["cycles_zero_faces"] = cycles0

    def _solve(self, r, f, warm_start: bool, p) -> None:
        st = _native.MGStats()
        self._ctx.call("gc_mg_solve", r.data_ptr(), f.data_ptr(), int(bool(warm_start)), C.byref(p), C.byref(st),
                       what="MultigridPoissonSolver.solve")
        self.last_cycles = int(st.cycles)
        self.last_stats = {
            "cycles": int(st.cycles),
            "converged": bool(st.converged),
            "rhs_norm": float(st.rhs_norm),
            "res_norm": float(st.res_norm),
            "rel_residual": float(st.res_norm / st.rhs_norm) if st.rhs_norm > 0 else 0.0,
        }

    def residual_norm(self, phi=None) -> float:
        """L2 norm (FP64) of the finest residual of the last solve.

        With ``phi`` given, the residual of that f32 potential; otherwise that of
        the solver's internal double-float iterate.
        """
        out = C.c_double()
        ptr = None
        if phi is not None:
            G = self.grid_size
            ptr = as_tensor(phi, shape=(G, G, G), name="phi").data_ptr()
        self._ctx.call("gc_mg_residual_norm", ptr, C.byref(out), what="residual_norm")
        return float(out.value)

    def moments(self, rho):
        """Raw FP64 moments [M, Smx, Smy, Smz, Smx2, Smy2, Smz2, Smxy, Smxz, Smyz] of rho."""
        G = self.grid_size
        r = as_tensor(rho, shape=(G, G, G), name="rho")
        out = (C.c_double * 10)()
        self._ctx.call("gc_moments", r.data_ptr(), out, what="moments")
        return list(out)

    def _moments_device(self, rho):
        """(M, CM, S_ab) from the device moments, as multigrid.py:364-389 returns them."""
        s = self.moments(rho)
        total = s[0]
        if total <= 0.0:
            return 0.0, (0.0, 0.0, 0.0), (0.0,) * 6
        cx, cy, cz = s[1] / total, s[2] / total, s[3] / total
        return total, (cx, cy, cz), (
            s[4] - total * cx * cx, s[5] - total * cy * cy, s[6] - total * cz * cz,
            s[7] - total * cx * cy, s[8] - total * cx * cz, s[9] - total * cy * cz,
        )


__all__ = ["MultigridPoissonSolver"]

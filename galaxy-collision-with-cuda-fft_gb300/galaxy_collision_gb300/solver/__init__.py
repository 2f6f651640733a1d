"""Poisson solvers behind the reference's factory (src/galaxy_collision/solver/__init__.py:12-22).

``make_solver('multigrid', G, **kw)`` returns the GB300 multigrid;
``make_solver('fft', G, **kw)`` the zero-padded isolated-Green FFT solver (FP64,
on the GPU through torch.fft), kept, as in the reference, to validate the
multigrid.
"""

from galaxy_collision_gb300.solver.base import PoissonSolver


def make_solver(name: str, grid_size: int, **kwargs) -> PoissonSolver:
    """Construct a solver by config name ('multigrid' or 'fft')."""
    if name == "multigrid":
        from galaxy_collision_gb300.solver.multigrid import MultigridPoissonSolver

        return MultigridPoissonSolver(grid_size, **kwargs)
    if name == "fft":
        from galaxy_collision_gb300.solver.fft import FFTPoissonSolver

        return FFTPoissonSolver(grid_size, **kwargs)
    raise ValueError(f"unknown solver {name!r} (expected 'multigrid' or 'fft')")


__all__ = ["PoissonSolver", "make_solver"]

"""The pluggable Poisson-solver interface (reference src/galaxy_collision/solver/base.py:27-41).

A solver maps a mass density ``rho`` to the potential ``phi`` solving
laplacian(phi) = 4 pi G rho with open (isolated) boundary conditions, on the
node-centred grid (node (i,j,k) at (i,j,k)*dx). ``solve`` reads ``rho`` and
overwrites ``phi`` in place; with ``warm_start`` an iterative solver may use the
current ``phi`` as its initial guess.
"""

from __future__ import annotations

from abc import ABC, abstractmethod


class PoissonSolver(ABC):
    """Maps mass density -> gravitational potential (laplacian phi = 4 pi G rho, open BCs)."""

    grid_size: int
    dx: float

    @abstractmethod
    def solve(self, rho, phi, warm_start: bool = False) -> None:
        raise NotImplementedError


__all__ = ["PoissonSolver"]

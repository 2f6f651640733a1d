"""Zero-padded isolated-Green's-function FFT Poisson solver (FP64, on the GPU).

Drop-in for ``FFTPoissonSolver`` (src/galaxy_collision/solver/fft_oracle.py:54-109):
the potential is the linear convolution of rho with g = -G dx^3 / r (self term 0),
done by FFT on a (pad_factor*G)^3 zero-padded grid so there are no periodic
images. The transforms are cuFFT calls through ``torch.fft`` in float64; this
solver validates the multigrid and measures its force error, it is not the
production solve.

``green="lattice"`` (an addition; the reference has only the continuum kernel)
convolves with the lattice Green's function of the 7-point Laplacian instead
(``solver/lattice_green.py``): the exact free-space solution of the discrete
problem the multigrid solves, which separates the multigrid's boundary and
solver error from the discretisation error of the 7-point stencil.
"""

from __future__ import annotations

import torch

from galaxy_collision_gb300 import units
from galaxy_collision_gb300.data import as_tensor
from galaxy_collision_gb300.solver.base import PoissonSolver


class FFTPoissonSolver(PoissonSolver):
    def __init__(self, grid_size: int, dx: float = 1.0, pad_factor: int = 2, grav_constant: float | None = None,
                 use_gpu: bool | None = None, *, green: str = "continuum"):
        if pad_factor < 2:
            raise ValueError(f"pad_factor must be >= 2 to avoid circular wrap, got {pad_factor}")
        self.grid_size = int(grid_size)
        self.dx = float(dx)
        self.pad = int(pad_factor) * self.grid_size
        self.G = units.G if grav_constant is None else float(grav_constant)
        if use_gpu is False:
            raise ValueError("this FFTPoissonSolver runs on the GPU only")
        if green not in ("continuum", "lattice"):
            raise ValueError(f"unknown Green's function {green!r} (expected 'continuum' or 'lattice')")
        self.green = green
        self._greens_ft = None

    def _green(self, device):
        if self._greens_ft is None and self.green == "lattice":
            from galaxy_collision_gb300.solver.lattice_green import lattice_green_kernel

            # phi = -(4 pi G / dx) (g * m), m = rho dx^3: L phi / dx^2 = 4 pi G rho
            ker = lattice_green_kernel(self.pad, device)
            ker *= -4.0 * 3.141592653589793 * self.G * self.dx**2
            self._greens_ft = torch.fft.rfftn(ker)
            del ker
        if self._greens_ft is None:
            m = self.pad
            a = torch.arange(m, device=device, dtype=torch.float64)
            d = torch.minimum(a, m - a)
            d2 = d * d
            r2 = d2[:, None, None] + d2[None, :, None] + d2[None, None, :]
            r2[0, 0, 0] = 1.0
            green = (-self.G * self.dx**3 / self.dx) / torch.sqrt(r2)
            green[0, 0, 0] = 0.0
            self._greens_ft = torch.fft.rfftn(green)
        return self._greens_ft

    def potential64(self, rho) -> torch.Tensor:
        """The FP64 potential (G^3) of rho (f32, or an FP64 CUDA tensor), without
        rounding to f32."""
        n, m = self.grid_size, self.pad
        if isinstance(rho, torch.Tensor) and rho.dtype == torch.float64:
            r = as_tensor(rho, dtype=torch.float64, shape=(n, n, n), name="rho")
        else:
            r = as_tensor(rho, shape=(n, n, n), name="rho")
        padded = torch.zeros((m, m, m), dtype=torch.float64, device=r.device)
        padded[:n, :n, :n] = r.to(torch.float64)
        spec = torch.fft.rfftn(padded) * self._green(r.device)
        del padded
        conv = torch.fft.irfftn(spec, s=(m, m, m))
        return conv[:n, :n, :n].contiguous()

    def solve(self, rho, phi, warm_start: bool = False) -> None:
        n = self.grid_size
        out = as_tensor(phi, shape=(n, n, n), name="phi")
        out.copy_(self.potential64(rho).to(torch.float32))


__all__ = ["FFTPoissonSolver"]

"""NumPy restatement of the reference's FFT oracle (test infrastructure only).

src/galaxy_collision/solver/fft_oracle.py:54-109: potential = linear
convolution of rho with g = -G dx^3 / r (r in node spacings times dx, self term
0), by rfftn on a zero-padded (pad*G)^3 grid. Everything in float64.
"""

from __future__ import annotations

import numpy as np


class FFTOracle:
    def __init__(self, grid_size, dx=1.0, pad_factor=2, grav_constant=1.0):
        if pad_factor < 2:
            raise ValueError(f"pad_factor must be >= 2 to avoid circular wrap, got {pad_factor}")
        self.grid_size = int(grid_size)
        self.dx = float(dx)
        self.pad = int(pad_factor) * self.grid_size
        self.G = float(grav_constant)
        m = self.pad
        d = np.minimum(np.arange(m), m - np.arange(m)).astype(np.float64)
        d2 = d * d
        r2 = d2[:, None, None] + d2[None, :, None] + d2[None, None, :]
        r2[0, 0, 0] = 1.0
        green = (-self.G * self.dx**3 / self.dx) / np.sqrt(r2)
        green[0, 0, 0] = 0.0
        self._gft = np.fft.rfftn(green)

    def potential(self, rho) -> np.ndarray:
        n, m = self.grid_size, self.pad
        padded = np.zeros((m, m, m), np.float64)
        padded[:n, :n, :n] = np.asarray(rho, dtype=np.float64)
        conv = np.fft.irfftn(np.fft.rfftn(padded) * self._gft, s=(m, m, m), axes=(0, 1, 2))
        return np.ascontiguousarray(conv[:n, :n, :n])

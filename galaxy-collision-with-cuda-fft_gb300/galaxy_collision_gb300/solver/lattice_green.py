"""Lattice Green's function of the 7-point Laplacian, for the FP64 FFT solver.

The reference's FFT solver convolves rho with the continuum kernel -G dx^3 / r
(src/galaxy_collision/solver/fft_oracle.py:82-96). The multigrid (the
reference's and this one) solves the 7-point discrete Laplacian, whose exact
free-space solution is the convolution with the lattice Green's function

    g(n) = (2 pi)^-3 int_BZ cos(k.n) / sum_i 2 (1 - cos k_i) d^3k ,   L g = -delta,

L f(n) = sum of the six neighbours - 6 f(n). With this kernel the FFT solver
gives the potential the multigrid converges to apart from its boundary (the
free-space potential instead of the multipole faces), so the difference of the
two separates the boundary error from the discretisation error that the
continuum kernel mixes in.

g is evaluated from the heat-kernel form g(n) = int_0^inf prod_i e^{-2t} I_{n_i}(2t)
dt: trapezoid rule in u = ln t (the integrand is smooth and bell-shaped in u
for every n) up to t_e ~ 4e8 with the Euler-Maclaurin end term, and the rest
from the large-t expansion prod_i (4 pi t)^{-1/2} (1 - (4 n_i^2 - 1)/(16 t)).
Only the wedge a >= b >= c is computed (g is symmetric under permutations and
sign changes of n); the table is built once per size on the host in float64
(one matrix product per first index).
"""

from __future__ import annotations

import functools

import numpy as np
from scipy.special import ive


@functools.lru_cache(maxsize=4)
def lattice_green_wedge(n: int) -> np.ndarray:
    """g[a, b, c] for 0 <= b, c <= a < n (float64); entries with b or c above a
    are left zero: look g(n) up at its indices sorted in descending order."""
    h = 0.05
    u = np.arange(np.log(1e-14), np.log(4e8), h)
    t = np.exp(u)
    w = h * t
    w[0] *= 0.5
    w[-1] *= 0.5
    k = np.arange(n)
    e = ive(k[:, None], 2.0 * t[None, :])  # e^{-2t} I_k(2t), (n, Q)
    te = t[-1]
    c0 = (4.0 * np.pi) ** -1.5
    q = (4.0 * k.astype(np.float64) ** 2 - 1.0) / 16.0
    g = np.zeros((n, n, n))
    for a in range(n):
        wa = e[a] * w
        blk = (e[: a + 1] * wa[None, :]) @ e[: a + 1].T  # (b, c), b, c <= a
        A = q[a] + q[: a + 1, None] + q[None, : a + 1]
        blk += c0 * (2.0 * te**-0.5 - (2.0 / 3.0) * A * te**-1.5)  # the tail [te, inf)
        blk += -(h * h / 12.0) * c0 * te**-0.5 * (-0.5 + 1.5 * A / te)  # end correction
        g[a, : a + 1, : a + 1] = blk
    return g


def lattice_green_table(n: int) -> np.ndarray:
    """The full table g[a, b, c], 0 <= a, b, c < n (for small n)."""
    g = lattice_green_wedge(n)
    k = np.arange(n)
    i, j, l = np.meshgrid(k, k, k, indexing="ij")
    s = np.stack([i, j, l])
    hi, lo = s.max(axis=0), s.min(axis=0)
    return g[hi, s.sum(axis=0) - hi - lo, lo]


def lattice_green_kernel(m: int, device) -> "torch.Tensor":
    """The periodic m^3 kernel of a zero-padded convolution, g(min(i, m-i), ...),
    built on the device plane by plane from the wedge (float64)."""
    import torch

    wedge = torch.from_numpy(lattice_green_wedge(m // 2 + 1)).to(device)
    n = wedge.shape[0]
    d = torch.arange(m, device=device)
    d = torch.minimum(d, m - d)
    dj, dk = torch.meshgrid(d, d, indexing="ij")
    flat = wedge.reshape(-1)
    out = torch.empty((m, m, m), dtype=torch.float64, device=device)
    for i in range(m):
        di = torch.full_like(dj, min(i, m - i))
        hi = torch.maximum(torch.maximum(di, dj), dk)
        lo = torch.minimum(torch.minimum(di, dj), dk)
        mid = di + dj + dk - hi - lo
        out[i] = flat[(hi * n + mid) * n + lo]
    return out


__all__ = ["lattice_green_wedge", "lattice_green_table", "lattice_green_kernel"]

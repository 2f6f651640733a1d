"""FP64 lattice Green's function of the 7-point Laplacian (test infrastructure only).

The reference validates its potential against an FP64 zero-padded FFT
convolution with the continuum kernel -G dx^3 / r, self term 0
(src/galaxy_collision/solver/fft_oracle.py:82-96). The reference's solver (and
this one) solves the 7-point discrete Laplacian, whose free-space solution is
the convolution with the lattice Green's function instead; against the
continuum kernel the two differ by the discretisation, not by the solver. This
module gives the commensurate oracle:

    g(n) = sum_{k in BZ} cos(k.n) / sum_i 2 (1 - cos k_i)     (so  L g = -delta,
           L f(n) = sum of the 6 neighbours - 6 f(n)),

computed from its heat-kernel form g(n) = int_0^inf prod_i e^{-2t} I_{n_i}(2t) dt
(the 1-D kernel of f(n+1) + f(n-1) - 2 f(n) is e^{-2t} I_n(2t)). The integral is
taken by the trapezoid rule in u = ln t on [ln 1e-14, ~ln 4e8] with the
Euler-Maclaurin end correction, and the rest [t_end, inf) analytically from
the large-t expansion e^{-x} I_n(x) = (2 pi x)^{-1/2} (1 - (4 n^2 - 1)/(8 x)). For
a table of N^3 offsets the quadrature is N matrix products. Accuracy: g(0)
equals Watson's constant 0.2527310098586625 to ~1e-14 and L g = -delta holds to
~1e-14 (tests/test_oracle_lattice_green.py).

Potential: phi = -(4 pi G / dx) (g * m), m = rho dx^3 per node, by a zero-padded
(2G)^3 FFT in float64 (the reference's padding, fft_oracle.py:70-71); far from
the mass g -> 1/(4 pi |n|), so phi -> -G M / r.
"""

from __future__ import annotations

import numpy as np
from scipy.special import ive

WATSON_G0 = 0.2527310098586625  # g(0) of the simple cubic lattice


def lgf_table(n: int, h_u: float = 0.05) -> np.ndarray:
    """g[a, b, c] for 0 <= a, b, c < n (the function is even in each index)."""
    u = np.arange(np.log(1e-14), np.log(4e8), h_u)
    t = np.exp(u)
    w = h_u * t
    w[0] *= 0.5
    w[-1] *= 0.5
    idx = np.arange(n)
    tab = ive(idx[:, None], 2.0 * t[None, :])  # e^{-2t} I_a(2t)
    g = np.empty((n, n, n))
    for a in range(n):
        g[a] = (tab[a][None, :] * w[None, :] * tab) @ tab.T
    q = 4.0 * idx.astype(np.float64) ** 2 - 1.0
    A = (q[:, None, None] + q[None, :, None] + q[None, None, :]) / 16.0
    te = t[-1]
    c = (4.0 * np.pi) ** -1.5
    g += c * (2.0 * te**-0.5 - (2.0 / 3.0) * A * te**-1.5)      # the tail [te, inf)
    g += -(h_u**2 / 12.0) * c * te**-0.5 * (-0.5 + 1.5 * A / te)  # end correction
    return g


def lgf_kernel(m: int) -> np.ndarray:
    """The (m)^3 periodic kernel of a zero-padded convolution: g(min(i, m - i), ...)."""
    half = m // 2
    g = lgf_table(half + 1)
    i = np.arange(m)
    i = np.minimum(i, m - i)
    return g[i[:, None, None], i[None, :, None], i[None, None, :]]


def lgf_potential(rho, dx: float, grav: float, pad_factor: int = 2) -> np.ndarray:
    """Free-space potential of the 7-point Laplacian: L phi / dx^2 = 4 pi G rho on
    the whole lattice, phi -> 0 at infinity, for rho on a G^3 node grid."""
    rho = np.asarray(rho, dtype=np.float64)
    G = rho.shape[0]
    m = pad_factor * G
    mass = np.zeros((m, m, m))
    mass[:G, :G, :G] = rho * dx**3
    ker = lgf_kernel(m)
    axes = (0, 1, 2)
    conv = np.fft.irfftn(np.fft.rfftn(mass, axes=axes) * np.fft.rfftn(ker, axes=axes), s=(m, m, m), axes=axes)
    return -(4.0 * np.pi * grav / dx) * np.ascontiguousarray(conv[:G, :G, :G])

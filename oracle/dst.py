"""Exact FP64 solution of the discrete Dirichlet problem (test infrastructure only).

Solves L phi = rhs on the interior of a G^3 node grid, L the 7-point Laplacian
with spacing dx, phi given on the six faces -- the discrete problem whose
solution the reference multigrid (and the GPU multigrid) converge to
(src/galaxy_collision/solver/multigrid.py:8-15). The face values move to the
right-hand side; the homogeneous interior problem is diagonal in the type-I
sine basis (scipy.fft.dstn, type=1).
"""

from __future__ import annotations

import numpy as np
from scipy.fft import dstn, idstn


def multipole_faces64(rho, dx, grav):
    """Monopole + quadrupole faces of rho about its centre of mass, in FP64
    (the formula of multigrid.py:261-295 and the moments of :364-389). The
    moments come from marginal sums of m = rho dx^3 (exact rearrangements of the
    triple sums), and the formula is evaluated on the 6 G^2 face nodes only."""
    rho = np.asarray(rho, dtype=np.float64)
    G = rho.shape[0]
    m = rho * dx**3
    ax = np.arange(G) * dx
    phi = np.zeros((G, G, G))
    M = m.sum()
    if M <= 0:
        return phi
    m_i, m_j, m_k = m.sum(axis=(1, 2)), m.sum(axis=(0, 2)), m.sum(axis=(0, 1))
    m_ij, m_ik, m_jk = m.sum(axis=2), m.sum(axis=1), m.sum(axis=0)
    c = np.array([ax @ m_i, ax @ m_j, ax @ m_k]) / M
    # raw second moments, then the parallel-axis shift to the centre of mass
    raw = np.empty((3, 3))
    raw[0, 0], raw[1, 1], raw[2, 2] = (ax * ax) @ m_i, (ax * ax) @ m_j, (ax * ax) @ m_k
    raw[0, 1] = raw[1, 0] = ax @ m_ij @ ax
    raw[0, 2] = raw[2, 0] = ax @ m_ik @ ax
    raw[1, 2] = raw[2, 1] = ax @ m_jk @ ax
    S = raw - M * np.outer(c, c)
    tr = np.trace(S)
    u, v = np.meshgrid(ax, ax, indexing="ij")
    e0, e1 = np.zeros_like(u), np.full_like(u, ax[-1])
    # (face slice, x, y, z of its nodes)
    faces = [((0, slice(None), slice(None)), e0, u, v), ((G - 1, slice(None), slice(None)), e1, u, v),
             ((slice(None), 0, slice(None)), u, e0, v), ((slice(None), G - 1, slice(None)), u, e1, v),
             ((slice(None), slice(None), 0), u, v, e0), ((slice(None), slice(None), G - 1), u, v, e1)]
    for sl, X, Y, Z in faces:
        rx, ry, rz = X - c[0], Y - c[1], Z - c[2]
        d2 = rx * rx + ry * ry + rz * rz + 1e-12
        d = np.sqrt(d2)
        nv = (rx / d, ry / d, rz / d)
        nsn = sum(nv[a] * S[a, b] * nv[b] for a in range(3) for b in range(3))
        phi[sl] = -grav * (M / d + (3.0 * nsn - tr) / (2.0 * d2 * d))
    return phi


def solve_dirichlet(rhs, faces, dx):
    """phi with phi = faces on the boundary and L phi = rhs (f64) on the interior."""
    rhs = np.asarray(rhs, dtype=np.float64)
    G = rhs.shape[0]
    phi = np.array(faces, dtype=np.float64, copy=True)
    phi[1:-1, 1:-1, 1:-1] = 0.0
    # move the boundary contribution to the right-hand side
    b = rhs[1:-1, 1:-1, 1:-1].copy()
    inv = 1.0 / dx**2
    b -= inv * (phi[2:, 1:-1, 1:-1] + phi[:-2, 1:-1, 1:-1] + phi[1:-1, 2:, 1:-1] + phi[1:-1, :-2, 1:-1]
                + phi[1:-1, 1:-1, 2:] + phi[1:-1, 1:-1, :-2])
    n = G - 2
    k = np.arange(1, n + 1)
    lam1 = (2.0 * np.cos(np.pi * k / (n + 1)) - 2.0) * inv
    lam = lam1[:, None, None] + lam1[None, :, None] + lam1[None, None, :]
    bh = dstn(b, type=1, workers=-1)
    u = idstn(bh / lam, type=1, workers=-1)
    phi[1:-1, 1:-1, 1:-1] = u
    return phi


def solve_reference_problem(rho, dx, grav):
    """FP64 exact solution of the reference's discrete problem for f32 density rho:
    rhs = f32(4 pi G) * rho (in f32, multigrid.py:463), FP64 multipole faces."""
    rho32 = np.asarray(rho, dtype=np.float32)
    rhs = (np.float32(4.0 * np.pi * grav) * rho32).astype(np.float64)
    faces = multipole_faces64(rho32, dx, grav)
    return solve_dirichlet(rhs, faces, dx)

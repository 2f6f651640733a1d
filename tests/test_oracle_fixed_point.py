"""The fixed-point deposit oracle (oracle/pm_oracle.c: or_deposit_fixed), pinned
by an independent NumPy restatement of its rule and by its defining properties.

The GPU deposit is tested bit for bit against or_deposit_fixed; this file pins
that oracle itself: per particle the reference's cell and weights in f32
(deposit.py:62-82), the partial product b = (m/dx^3 * wx) * wy in f32, every
corner the exact product b * wz rounded once to the nearest multiple of the
quantum 2^E (ties to even), summed in int64; E from the exact, order-independent
total mass. The quantised density is then independent of the particle order,
conserves the quanta exactly, and is within half a quantum per contribution of
the FP64 sum of the reference's f32 contributions.
"""

from __future__ import annotations

import numpy as np
import pytest

from oracle import pm


def _restated(pos, mass, dx, G, bits):
    """NumPy restatement of the fixed-point rule (small inputs)."""
    f32 = np.float32
    dx = f32(dx)
    inv_vol = f32(1.0) / (dx * dx * dx)
    mm = (mass.astype(f32) * inv_vol).astype(f32)
    n = pos.shape[0]
    # exact total: terms truncated to multiples of 2^-s, s from the largest term
    ok = np.isfinite(mm) & (mm > 0)
    maxbits = int(mm[ok].view(np.uint32).max()) if ok.any() else 0
    L = 0
    while (1 << L) < n:
        L += 1
    S = 0.0
    if maxbits:
        emax = ((maxbits >> 23) & 0xFF) - 127
        sh = 62 - L - (emax + 1)
        isum = sum(int(np.trunc(float(v) * 2.0**sh)) for v in mm[ok])
        S = isum * 2.0**-sh
    E = (np.frexp(S)[1] if S > 0 else 0) - bits
    E = max(-120, min(120, E))
    q = np.zeros((G, G, G), np.int64)
    g = (pos.astype(f32) / dx).astype(f32)
    for p in range(n):
        gx, gy, gz = g[p]
        if not (-1 <= gx < G and -1 <= gy < G and -1 <= gz < G):
            continue
        fl = np.floor(g[p]).astype(f32)
        f = (g[p] - fl).astype(f32)
        w = [(f32(1.0) - f[a], f[a]) for a in range(3)]
        ix, iy, iz = (int(v) for v in fl)
        for a in range(2):
            for b_ in range(2):
                b = f32(f32(mm[p] * w[0][a]) * w[1][b_])
                for c in range(2):
                    jx, jy, jz = ix + a, iy + b_, iz + c
                    if 0 <= jx < G and 0 <= jy < G and 0 <= jz < G:
                        q[jx, jy, jz] += int(np.rint(float(b) * float(w[2][c]) * 2.0**-E))
    return q, E


@pytest.mark.parametrize("dx,bits", [(1.0, 52), (0.375, 40), (2.5, 30)])
def test_fixed_point_oracle_equals_the_restated_rule(dx, bits):
    G = 12
    rng = np.random.default_rng(int(dx * 8) + bits)
    pos = rng.uniform(-1.5 * dx, (G + 0.5) * dx, size=(1500, 3)).astype(np.float32)
    pos[:5] = np.float32([[0, 0, 0], [dx * (G - 1), 1, 1], [-0.5 * dx, 2, 2], [dx * 3.5, dx * 3.5, dx * 3.5],
                          [-dx, dx, dx]])
    mass = rng.uniform(0.1, 3.0, size=pos.shape[0]).astype(np.float32)
    _, q, E = pm.deposit_fixed(pos, mass, dx, G, bits)
    q_ref, E_ref = _restated(pos, mass, dx, G, bits)
    assert E == E_ref
    np.testing.assert_array_equal(q, q_ref)


def test_fixed_point_oracle_is_order_independent_and_near_the_fp64_sum():
    G, dx, bits = 16, 0.5, 44
    rng = np.random.default_rng(3)
    pos = rng.normal(4.0, 1.2, size=(20000, 3)).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, size=pos.shape[0]).astype(np.float32)
    rho, q, E = pm.deposit_fixed(pos, mass, dx, G, bits)
    perm = rng.permutation(pos.shape[0])
    rho2, q2, E2 = pm.deposit_fixed(pos[perm], mass[perm], dx, G, bits)
    assert E2 == E
    np.testing.assert_array_equal(q, q2)
    np.testing.assert_array_equal(rho, rho2)
    # each corner is its exact product rounded to the quantum: the node sums are
    # within half a quantum per contribution of the FP64 sum of f32 contributions
    # (the f32 rounding of the last product is below the quantum at these sizes)
    ref = pm.deposit_f64(pos, mass, dx, G)
    counts = np.zeros((G, G, G), np.int64)
    g = np.floor(pos / np.float32(dx)).astype(np.int64)
    for a in range(2):
        for b in range(2):
            for c in range(2):
                j = g + np.array([a, b, c])
                keep = np.all((j >= 0) & (j < G), axis=1) & np.all((g >= -1) & (g < G), axis=1)
                np.add.at(counts, (j[keep, 0], j[keep, 1], j[keep, 2]), 1)
    quantum = 2.0**E
    f32_err = np.abs(ref) * 2.0**-23  # the f32 rounding of the reference's contributions
    assert np.all(np.abs(q * quantum - ref) <= counts * (0.5 * quantum) + f32_err + 1e-300)

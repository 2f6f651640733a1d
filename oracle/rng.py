"""Philox4x32-10 restated in NumPy (test infrastructure only).

The device initial-condition samplers draw their random numbers from the
counter-based generator of Salmon, Moraes, Dror and Shaw ("Parallel random
numbers: as easy as 1, 2, 3", SC 2011). This is the same published algorithm,
vectorised over counters, used to check the device generator bit for bit and
to check the uniforms' distribution. The reference has no device generator
(it samples with NumPy on the host), so parity is pinned to the algorithm.
"""

from __future__ import annotations

import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c = [np.asarray(v, np.uint32).copy() for v in (c0, c1, c2, c3)]
    k0, k1 = np.uint32(k0), np.uint32(k1)
    with np.errstate(over="ignore"):
        for _ in range(10):
            p0 = M0 * c[0].astype(np.uint64)
            p1 = M1 * c[2].astype(np.uint64)
            hi0, lo0 = (p0 >> np.uint64(32)).astype(np.uint32), (p0 & MASK).astype(np.uint32)
            hi1, lo1 = (p1 >> np.uint64(32)).astype(np.uint32), (p1 & MASK).astype(np.uint32)
            c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
            k0 = np.uint32((int(k0) + int(W0)) & 0xFFFFFFFF)
            k1 = np.uint32((int(k1) + int(W1)) & 0xFFFFFFFF)
    return c


def u01(b):
    """Uniform f32 in (0, 1) from the top 24 bits, centred in its bin."""
    return ((np.asarray(b, np.uint32) >> np.uint32(8)).astype(np.float32) + np.float32(0.5)) * np.float32(
        1.0 / 16777216.0)


def uniforms(seed: int, stream: int, n: int) -> np.ndarray:
    """(n, 4) uniforms of counters (i, 0, stream) for i < n, key = seed."""
    i = np.arange(n, dtype=np.uint64)
    c = philox4x32_10((i & MASK).astype(np.uint32), (i >> np.uint64(32)).astype(np.uint32),
                      np.zeros(n, np.uint32), np.full(n, stream, np.uint32), seed & 0xFFFFFFFF, seed >> 32)
    return np.stack([u01(v) for v in c], axis=1)


__all__ = ["philox4x32_10", "u01", "uniforms"]

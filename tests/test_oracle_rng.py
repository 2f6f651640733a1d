"""The NumPy restatement of Philox4x32-10 (the device IC generator) draws
uniforms that look uniform and independent across streams and keys."""

from __future__ import annotations

import numpy as np

from oracle import rng


def test_uniforms_in_open_interval_and_flat():
    u = rng.uniforms(1234, 5, 50000).ravel()
    assert u.min() > 0.0 and u.max() < 1.0
    counts, _ = np.histogram(u, bins=64, range=(0.0, 1.0))
    expected = u.size / 64
    chi2 = float(((counts - expected) ** 2 / expected).sum())
    assert chi2 < 120.0  # 63 degrees of freedom: p ~ 1e-5 at 120
    assert abs(u.mean() - 0.5) < 5 / np.sqrt(12 * u.size)


def test_streams_and_keys_decorrelate():
    a = rng.uniforms(7, 0, 20000)[:, 0]
    b = rng.uniforms(7, 1, 20000)[:, 0]
    c = rng.uniforms(8, 0, 20000)[:, 0]
    for x, y in ((a, b), (a, c)):
        assert abs(np.corrcoef(x, y)[0, 1]) < 0.03
    # a counter step changes about half the output bits
    w = rng.philox4x32_10(np.arange(2000, dtype=np.uint32), 0, 0, 0, 1, 2)[0]
    flips = np.unpackbits((w[1:] ^ w[:-1]).view(np.uint8)).mean()
    assert 0.45 < flips < 0.55

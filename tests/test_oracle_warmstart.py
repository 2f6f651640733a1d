"""The warm-start network's CPU oracle: its backward pass against finite differences.

The oracle (float64, no bf16 rounding) is the yardstick for the tensor-core
forward/backward kernels, so its own gradient is checked first: central
differences of the loss 0.5 mean((y - t)^2) on sampled parameters of every layer.
"""

from __future__ import annotations

import numpy as np

from oracle import warmstart as ows


def _params(seed):
    rng = np.random.default_rng(seed)
    out = []
    for i, (ci, co, _, _) in enumerate(ows.LAYERS):
        w = rng.normal(0.0, np.sqrt(2.0 / (27 * ci)), size=(27, co, ci))
        out += [w.ravel(), rng.normal(0.0, 0.05, size=co)]
    return np.concatenate(out)


def test_oracle_backward_matches_finite_differences():
    R = 16
    rng = np.random.default_rng(1)
    p = _params(2)
    feat = rng.normal(size=(4, R, R, R))
    target = 0.1 * rng.normal(size=(R, R, R))
    y, cache = ows.forward(p, feat, emulate=False)
    loss, g = ows.backward(cache, target, emulate=False)
    assert loss == ows.loss_only(p, feat, target)
    off, checked, bad = 0, 0, []
    for li, (ci, co, _, _) in enumerate(ows.LAYERS):
        nw = 27 * ci * co
        idx = list(rng.choice(nw, size=3, replace=False) + off) + [off + nw + int(rng.integers(co))]
        for i in idx:
            e = 1e-5
            pp, pm = p.copy(), p.copy()
            pp[i] += e
            pm[i] -= e
            fd = (ows.loss_only(pp, feat, target) - ows.loss_only(pm, feat, target)) / (2 * e)
            checked += 1
            if abs(fd - g[i]) > 1e-7 + 1e-4 * abs(g[i]):
                bad.append((li, i, fd, g[i]))
        off += nw + co
    # a ReLU kink inside the difference stencil may spoil one sample, not more
    assert len(bad) <= 1, bad
    assert checked == 4 * len(ows.LAYERS)


def test_oracle_adjoint_identities():
    """<conv x, g> = <x, dgrad g> and <pool x, g> = <x, up(g)/8>, <up x, g> = <x, up_adjoint g>."""
    rng = np.random.default_rng(3)
    R = 8
    x = rng.normal(size=(16, R, R, R))
    g = rng.normal(size=(32, R, R, R))
    W = rng.normal(size=(27, 32, 16))
    assert np.isclose(np.sum(ows.conv(x, W) * g), np.sum(x * ows.conv_dgrad(g, W)), rtol=1e-10)
    dW = ows.conv_wgrad(x, g)
    assert np.isclose(np.sum(ows.conv(x, W) * g), np.sum(W * dW), rtol=1e-10)
    h = rng.normal(size=(16, R // 2, R // 2, R // 2))
    assert np.isclose(np.sum(ows.pool(x) * h), np.sum(x * ows.up(h) / 8.0), rtol=1e-10)
    assert np.isclose(np.sum(ows.up(h) * x), np.sum(h * ows.up_adjoint(x)), rtol=1e-10)


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2**-8, 1.0 + 3 * 2**-9, -2.5, 3.0e38, np.inf], np.float32)
    r = ows.bf16(v)
    assert r[0] == 1.0 and r[1] == 1.0  # tie -> even
    assert r[2] == 1.0 + 2**-7          # above the tie
    assert r[3] == -2.5 and np.isinf(r[5])

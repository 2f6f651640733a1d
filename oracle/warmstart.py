"""CPU oracle of the learned warm-start network (test infrastructure only).

The reference has no learned component: its multigrid starts from the previous
potential (src/galaxy_collision/solver/multigrid.py:464-467). This module
restates, in NumPy, the network the GPU trains and runs in its place, so the
tensor-core forward and backward passes can be checked:

* ``forward``/``backward`` with ``emulate=True`` round weights and stored
  activations to bf16 (round to nearest even) at the same points as the device
  kernels and accumulate in float64; the device accumulates in float32, so the
  two agree to bf16 resolution, not bit for bit;
* with ``emulate=False`` everything is float64, which is what the finite-
  difference check of the backward pass uses.

Arrays are [channel][z][y][x] (x fastest, the device voxel order); tap
t = (dz+1)*9 + (dy+1)*3 + (dx+1); parameters are the flat vector of
``galaxy_collision_gb300.warmstart`` (per layer W[27][cout][cin] then b[cout]).
Parity pinned to the network definition only: no reference test covers it.
"""

from __future__ import annotations

import numpy as np

LAYERS = [(16, 16, 0, 1), (16, 32, 1, 1), (32, 64, 2, 1), (64, 128, 3, 1), (128, 64, 3, 0), (64, 64, 2, 1),
          (64, 32, 2, 0), (32, 32, 1, 1), (32, 16, 1, 0), (16, 16, 0, 1), (16, 16, 0, 0)]


def bf16(a):
    """Round float32 values to bf16 (nearest even), returned as float64."""
    u = np.asarray(a, np.float32).view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    r = np.where(nan, np.uint32(0x7FC00000), r)
    return r.view(np.float32).astype(np.float64)


def _ident(a):
    return np.asarray(a, np.float64)


def unpack(params, layers=LAYERS):
    out, off = [], 0
    for ci, co, _, _ in layers:
        W = np.asarray(params[off:off + 27 * co * ci], np.float64).reshape(27, co, ci)
        off += 27 * co * ci
        b = np.asarray(params[off:off + co], np.float64)
        off += co
        out.append((W, b))
    return out


def _taps():
    for t in range(27):
        yield t, t // 9 - 1, (t // 3) % 3 - 1, t % 3 - 1


def conv(x, W, b=None):
    """out[co][v] = sum_t sum_ci x[ci][v + off_t] W[t][co][ci] (+ b[co]), zero padding."""
    R = x.shape[1]
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1)))
    out = np.zeros((W.shape[1], R, R, R))
    for t, dz, dy, dx in _taps():
        sh = xp[:, 1 + dz:1 + dz + R, 1 + dy:1 + dy + R, 1 + dx:1 + dx + R]
        out += np.tensordot(W[t], sh, axes=([1], [0]))
    if b is not None:
        out += b[:, None, None, None]
    return out


def conv_dgrad(g, W):
    """Adjoint of conv in its input: gin[ci][v] = sum_t sum_co g[co][v - off_t] W[t][co][ci]."""
    R = g.shape[1]
    gp = np.pad(g, ((0, 0), (1, 1), (1, 1), (1, 1)))
    out = np.zeros((W.shape[2], R, R, R))
    for t, dz, dy, dx in _taps():
        sh = gp[:, 1 - dz:1 - dz + R, 1 - dy:1 - dy + R, 1 - dx:1 - dx + R]
        out += np.tensordot(W[t].T, sh, axes=([1], [0]))
    return out


def conv_wgrad(x, g):
    """dW[t][co][ci] = sum_v g[co][v] x[ci][v + off_t]."""
    R = x.shape[1]
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1)))
    dW = np.zeros((27, g.shape[0], x.shape[0]))
    for t, dz, dy, dx in _taps():
        sh = xp[:, 1 + dz:1 + dz + R, 1 + dy:1 + dy + R, 1 + dx:1 + dx + R]
        dW[t] = np.tensordot(g, sh, axes=([1, 2, 3], [1, 2, 3]))
    return dW


def pool(x):
    C, R = x.shape[0], x.shape[1]
    return x.reshape(C, R // 2, 2, R // 2, 2, R // 2, 2).mean(axis=(2, 4, 6))


def up(x):
    return x.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def up_adjoint(g):
    C, R = g.shape[0], g.shape[1]
    return g.reshape(C, R // 2, 2, R // 2, 2, R // 2, 2).sum(axis=(2, 4, 6))


def relu(x):
    return np.maximum(x, 0.0)


def forward(params, feat, emulate=True):
    """feat: (4, R, R, R) (float16 or float). Returns (y, cache)."""
    r = bf16 if emulate else _ident
    P = [(r(W.astype(np.float32)) if emulate else W, b) for W, b in unpack(params)]
    R = feat.shape[1]
    x0 = np.zeros((16, R, R, R))
    x0[:feat.shape[0]] = r(np.asarray(feat, np.float32))
    c = {"x0": x0, "P": P}
    c["e0"] = r(relu(conv(x0, *P[0])))
    c["p1"] = r(pool(c["e0"]))
    c["e1"] = r(relu(conv(c["p1"], *P[1])))
    c["p2"] = r(pool(c["e1"]))
    c["e2"] = r(relu(conv(c["p2"], *P[2])))
    c["p3"] = r(pool(c["e2"]))
    c["e3"] = r(relu(conv(c["p3"], *P[3])))
    c["u2"] = r(conv(c["e3"], *P[4]))
    c["d2"] = r(relu(up(c["u2"]) + c["e2"]))
    c["f2"] = r(relu(conv(c["d2"], *P[5])))
    c["u1"] = r(conv(c["f2"], *P[6]))
    c["d1"] = r(relu(up(c["u1"]) + c["e1"]))
    c["f1"] = r(relu(conv(c["d1"], *P[7])))
    c["u0"] = r(conv(c["f1"], *P[8]))
    c["d0"] = r(relu(up(c["u0"]) + c["e0"]))
    c["f0"] = r(relu(conv(c["d0"], *P[9])))
    y = conv(c["f0"], *P[10])[0]
    if emulate:
        y = y.astype(np.float32).astype(np.float64)
    c["y"] = y
    return y, c


def backward(c, target, emulate=True):
    """Loss 0.5 mean((y - target)^2) and the flat parameter gradient."""
    r = bf16 if emulate else _ident
    P = c["P"]
    y = c["y"]
    R = y.shape[0]
    n = float(R**3)
    d = y - np.asarray(target, np.float64)
    loss = 0.5 * float(np.mean(d * d))
    gy = np.zeros((16, R, R, R))
    gy[0] = r((d.astype(np.float32) * np.float32(1.0 / n))) if emulate else d / n
    grads = [None] * len(LAYERS)

    def lay(i, x, g):
        grads[i] = (conv_wgrad(x, g), g.sum(axis=(1, 2, 3)))

    mask = lambda g, a: np.where(a > 0, g, 0.0)  # noqa: E731
    lay(10, c["f0"], gy)
    g_f0 = r(mask(conv_dgrad(gy, P[10][0]), c["f0"]))
    lay(9, c["d0"], g_f0)
    g_d0 = r(mask(conv_dgrad(g_f0, P[9][0]), c["d0"]))
    g_u0 = r(up_adjoint(g_d0))
    lay(8, c["f1"], g_u0)
    g_f1 = r(mask(conv_dgrad(g_u0, P[8][0]), c["f1"]))
    lay(7, c["d1"], g_f1)
    g_d1 = r(mask(conv_dgrad(g_f1, P[7][0]), c["d1"]))
    g_u1 = r(up_adjoint(g_d1))
    lay(6, c["f2"], g_u1)
    g_f2 = r(mask(conv_dgrad(g_u1, P[6][0]), c["f2"]))
    lay(5, c["d2"], g_f2)
    g_d2 = r(mask(conv_dgrad(g_f2, P[5][0]), c["d2"]))
    g_u2 = r(up_adjoint(g_d2))
    lay(4, c["e3"], g_u2)
    g_e3 = r(mask(conv_dgrad(g_u2, P[4][0]), c["e3"]))
    lay(3, c["p3"], g_e3)
    g_p3 = r(conv_dgrad(g_e3, P[3][0]))
    g_e2 = r(mask(g_d2 + 0.125 * up(g_p3), c["e2"]))
    lay(2, c["p2"], g_e2)
    g_p2 = r(conv_dgrad(g_e2, P[2][0]))
    g_e1 = r(mask(g_d1 + 0.125 * up(g_p2), c["e1"]))
    lay(1, c["p1"], g_e1)
    g_p1 = r(conv_dgrad(g_e1, P[1][0]))
    g_e0 = r(mask(g_d0 + 0.125 * up(g_p1), c["e0"]))
    lay(0, c["x0"], g_e0)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat


def loss_only(params, feat, target, emulate=False):
    y, _ = forward(params, feat, emulate=emulate)
    d = y - np.asarray(target, np.float64)
    return 0.5 * float(np.mean(d * d))


__all__ = ["LAYERS", "bf16", "conv", "conv_dgrad", "conv_wgrad", "pool", "up", "up_adjoint", "forward", "backward",
           "loss_only", "unpack"]

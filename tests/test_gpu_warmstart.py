"""The learned warm start's tensor-core kernels against the CPU oracle.

* the single-tile tcgen05 GEMM for every operand major-ness (descriptor check);
* the network's forward pass and its parameter gradient (BF16 operands, FP32
  accumulation) against oracle/warmstart.py emulating the same bf16 roundings;
* a short Adam run that must fit a fixed target.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import warmstart as ows

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("N,K", [(16, 16), (64, 32), (128, 64), (256, 64)])
@pytest.mark.parametrize("a_mn,b_mn", [(0, 0), (1, 1), (0, 1), (1, 0)])
def test_tensor_core_tile_gemm(cuda, N, K, a_mn, b_mn):
    from galaxy_collision_gb300 import _native

    L = _native.lib()
    g = torch.Generator(device="cpu").manual_seed(N * 131 + K + 7 * a_mn + 3 * b_mn)
    A = torch.randn(128, K, generator=g).to(torch.bfloat16).cuda()
    B = torch.randn(N, K, generator=g).to(torch.bfloat16).cuda()
    D = torch.full((128, N), float("nan"), device="cuda")
    st = torch.zeros(1, dtype=torch.int32, device="cuda")
    rc = L.gc_ws_selftest_gemm(C.c_void_p(A.data_ptr()), C.c_void_p(B.data_ptr()), C.c_void_p(D.data_ptr()), N, K,
                               a_mn, b_mn, 0, _native.current_stream_handle(), C.c_void_p(st.data_ptr()))
    assert rc == 0
    torch.cuda.synchronize()
    assert int(st.item()) == 0
    ref = A.double() @ B.double().T
    assert torch.allclose(D.double(), ref, rtol=1e-5, atol=1e-4)


def _rand_params(seed):
    rng = np.random.default_rng(seed)
    out = []
    for ci, co, _, _ in ows.LAYERS:
        out += [rng.normal(0.0, np.sqrt(2.0 / (27 * ci)), size=(27, co, ci)).ravel(), rng.normal(0.0, 0.05, size=co)]
    return np.concatenate(out).astype(np.float32)


def _feat(R, seed):
    rng = np.random.default_rng(seed)
    return rng.normal(size=(4, R, R, R)).astype(np.float16)


@pytest.mark.parametrize("R", [16, 32])
def test_forward_matches_oracle(cuda, R):
    from galaxy_collision_gb300.warmstart import WarmStartNet

    p = _rand_params(R)
    feat = _feat(R, R + 1)
    net = WarmStartNet(R, params=p)
    y = net.forward(torch.from_numpy(feat).cuda()).cpu().numpy()
    assert net.status() == 0
    yo, _ = ows.forward(p, feat, emulate=True)
    assert rel_l2(y, yo) < 1e-2


def test_backward_matches_oracle(cuda):
    from galaxy_collision_gb300.warmstart import WarmStartNet, param_slices

    R = 16
    p = _rand_params(5)
    feat = _feat(R, 6)
    target = (0.1 * np.random.default_rng(7).normal(size=(R, R, R))).astype(np.float16)
    net = WarmStartNet(R, params=p)
    net.forward(torch.from_numpy(feat).cuda())
    loss = float(net.backward(torch.from_numpy(target).cuda()).item())
    g = net.grads().cpu().numpy()
    assert net.status() == 0
    _, cache = ows.forward(p, feat, emulate=True)
    lo, go = ows.backward(cache, target.astype(np.float64), emulate=True)
    assert loss == pytest.approx(lo, rel=1e-3)
    # bf16 activations and gradients are rounded at ~20 points; fp32 (device) and
    # fp64 (oracle) accumulation flip some of those roundings, so agreement is to
    # bf16 resolution: a few percent per layer, ~1% over the whole gradient
    assert rel_l2(g, go) < 2e-2
    for i, (ws, bs) in enumerate(param_slices()):
        assert rel_l2(g[ws], go[ws]) < 6e-2, f"layer {i} weights"
        assert rel_l2(g[bs], go[bs]) < 6e-2, f"layer {i} bias"
        cos = float(np.dot(g[ws], go[ws]) / (np.linalg.norm(g[ws]) * np.linalg.norm(go[ws])))
        assert cos > 0.998, f"layer {i} weights: cosine {cos}"


def test_autotuned_plans_keep_the_results(cuda):
    """The autotuner only changes tile shapes: forward and gradient still match
    the oracle after it has picked the fastest plans."""
    from galaxy_collision_gb300.warmstart import WarmStartNet

    R = 32
    p = _rand_params(8)
    feat = _feat(R, 9)
    target = (0.1 * np.random.default_rng(10).normal(size=(R, R, R))).astype(np.float16)
    net = WarmStartNet(R, params=p)
    ms = net.autotune(iters=2)
    assert ms.shape == (11, 3) and np.all(ms[:, 0] > 0) and np.all(ms[:, 2] > 0)
    assert all(len(row) == 3 for row in net.plans())
    y = net.forward(torch.from_numpy(feat).cuda()).cpu().numpy()
    net.backward(torch.from_numpy(target).cuda())
    g = net.grads().cpu().numpy()
    assert net.status() == 0
    yo, cache = ows.forward(p, feat, emulate=True)
    _, go = ows.backward(cache, target.astype(np.float64), emulate=True)
    assert rel_l2(y, yo) < 1e-2
    assert rel_l2(g, go) < 2e-2


def test_adam_fits_a_fixed_target(cuda):
    """A smooth target that depends on the inputs: 80 Adam steps on one sample."""
    from galaxy_collision_gb300.warmstart import WarmStartNet

    R = 32
    rng = np.random.default_rng(11)
    z, y, x = np.meshgrid(*[np.linspace(-1, 1, R)] * 3, indexing="ij")
    feat = np.stack([np.exp(-4 * (x**2 + y**2 + z**2)), x * y, np.sin(3 * z), x + z]).astype(np.float16)
    target = (0.5 * feat[0] - 0.3 * feat[2] + 0.05 * rng.normal(size=(R, R, R))).astype(np.float16)
    net = WarmStartNet(R, seed=3)
    f, t = torch.from_numpy(feat).cuda(), torch.from_numpy(target).cuda()
    losses = []
    for _ in range(80):
        net.forward(f)
        losses.append(float(net.backward(t).item()))
        net.adam_step(lr=3e-3)
    assert net.status() == 0
    assert losses[-1] < 0.3 * losses[0], losses[::10]


def _cluster(n, G, seed):
    rng = np.random.default_rng(seed)
    pos = (rng.normal(size=(n, 3)) * 3.0 + (G - 1) / 2.0).astype(np.float32)
    vel = (rng.normal(size=(n, 3)) * 0.3).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, size=n).astype(np.float32) / n
    return pos, vel, mass


def _coarse(phi):
    G = phi.shape[0]
    return phi.reshape(G // 2, 2, G // 2, 2, G // 2, 2).mean(axis=(1, 3, 5))


def test_engine_records_features_and_target(cuda):
    """The recorded sample: the step's features (coarse potential, its first and
    second differences, normalised) and the second difference its solve produced,
    in units of the previous second difference's rms."""
    from galaxy_collision_gb300.engine import PMEngine

    G, dt = 32, 0.05
    pos, vel, mass = _cluster(20000, G, 1)
    eng = PMEngine(G, 1.0, tol=1e-9, max_cycles=80, sort_every=0)
    eng.set_warmstart("plain", track=True)
    eng.load(pos, vel, mass)
    eng.prime(dt)
    phis = [eng.potential().double().cpu().numpy()]
    for _ in range(3):
        eng.advance(dt)
        phis.append(eng.potential().double().cpu().numpy())
    rec = torch.zeros((5, G // 2, G // 2, G // 2), dtype=torch.float16, device="cuda")
    eng.record_sample(rec)
    eng.advance(dt)
    phis.append(eng.potential().double().cpu().numpy())
    r = rec.float().cpu().numpy()
    c = [_coarse(p) for p in phis]
    d_prev, d_new = c[3] - c[2], c[4] - c[3]
    dd_prev, dd_new = d_prev - (c[2] - c[1]), d_new - d_prev
    rms = lambda a: np.sqrt(np.mean(a**2))  # noqa: E731
    assert np.all(np.isfinite(r))
    assert r[0].min() >= 0.0  # log(1 + rho / mean)
    np.testing.assert_allclose(r[1], c[3] / rms(c[3]), rtol=0, atol=2e-3 * np.abs(r[1]).max())
    np.testing.assert_allclose(r[2], d_prev / rms(d_prev), rtol=0, atol=3e-3 * np.abs(r[2]).max())
    np.testing.assert_allclose(r[3], dd_prev / rms(dd_prev), rtol=0, atol=2e-2 * np.abs(r[3]).max())
    np.testing.assert_allclose(r[4], dd_new / rms(dd_prev), rtol=0, atol=2e-2 * np.abs(r[4]).max() + 1e-3)


@pytest.mark.parametrize("mode", ["extrapolate", "learned"])
def test_warm_start_modes_reach_the_same_solution(cuda, mode):
    """Only the initial guess changes: trajectories agree with the plain warm start
    to the solver tolerance; an untrained network (zero output layer) is exactly
    the extrapolation."""
    from galaxy_collision_gb300.engine import PMEngine
    from galaxy_collision_gb300.warmstart import WarmStartNet

    G, dt, steps = 32, 0.05, 8
    pos, vel, mass = _cluster(30000, G, 2)

    def run(m, net=None):
        eng = PMEngine(G, 1.0, tol=1e-8, max_cycles=80, sort_every=0)
        eng.set_warmstart(m, net=net, track=True)
        eng.load(pos, vel, mass)
        eng.prime(dt)
        cyc = [eng.advance(dt).cycles for _ in range(steps)]
        eng.synchronize(dt)
        p, v, _, _ = eng.state_arrays()
        return p.cpu().numpy(), v.cpu().numpy(), cyc

    p0, v0, c0 = run("plain")
    net = WarmStartNet(G // 2, seed=0) if mode == "learned" else None
    p1, v1, c1 = run(mode, net)
    assert np.abs(p1 - p0).max() < 1e-5
    assert np.abs(v1 - v0).max() < 1e-5 * np.abs(v0).max() + 1e-7
    assert sum(c1) <= sum(c0)
    if mode == "learned":
        _, _, ce = run("extrapolate")
        assert c1 == ce
        assert net.status() == 0


def test_trained_network_gain(cuda):
    """What the shipped network adds to the method without it. On held-out
    collisions (seeds outside the training set) its prediction of the next second
    difference of the potential has a lower loss than predicting none (the linear
    extrapolation, the method without the network) and than repeating the last
    one; and with it the multigrid needs no more V-cycles than with the
    extrapolation, and fewer than from the previous potential (the reference's
    warm start)."""
    from galaxy_collision_gb300 import warmstart_train as wt
    from galaxy_collision_gb300.warmstart import WEIGHTS_PATH, WarmStartNet

    if not WEIGHTS_PATH.exists():
        pytest.skip("no trained weights shipped")
    net = WarmStartNet.load(WEIGHTS_PATH)
    val = wt.generate_samples(2, 1_000_000, 40, 10, seed=987_654)
    loss = wt.validation_loss(net, val)
    assert loss["network"] < 0.85 * loss["zero"], loss
    assert loss["network"] < loss["previous"], loss
    ev = wt.evaluate(net, 2_000_000, steps=6, seed=424_242, warm_steps=4)
    assert ev["learned"]["mean_vcycles"] <= ev["extrapolate"]["mean_vcycles"]
    assert ev["extrapolate"]["mean_vcycles"] < ev["plain"]["mean_vcycles"]
    assert net.status() == 0


@pytest.mark.parametrize("tol,dt", [(1e-6, 0.04), (1e-8, 0.02)])
def test_trained_network_removes_a_vcycle_at_large_steps(cuda, tol, dt):
    """Where the step-to-step change of the potential is large against the
    tolerance (a 4x or 8x larger time step than the configuration's 0.005, or a
    100x tighter tolerance), the network's correction leaves a smaller initial
    residual than the extrapolation alone: strictly fewer V-cycles per step on
    the 10M-particle two-disk collision at 256^3 (measured on GB300: 2 against 3
    at tol 1e-6, dt 0.04; 3 against 4 at tol 1e-8, dt 0.02). At the
    configuration's own dt and tolerance both need the minimum, one."""
    from galaxy_collision_gb300 import ic
    from galaxy_collision_gb300.engine import PMEngine
    from galaxy_collision_gb300.warmstart import WEIGHTS_PATH, WarmStartNet

    if not WEIGHTS_PATH.exists():
        pytest.skip("no trained weights shipped")
    net = WarmStartNet.load(WEIGHTS_PATH)
    icr, cfg = ic.build("two_disk_10M")
    cycles = {}
    for mode in ("extrapolate", "learned"):
        e = PMEngine(cfg["grid"], cfg["dx"], origin=cfg["origin"], tol=tol, max_cycles=80,
                     fixed_point_bits=cfg["fixed_point_bits"])
        e.set_warmstart(mode, net=net if mode == "learned" else None)
        e.load(icr.pos, icr.vel, icr.mass, icr.gid, sort=True)
        e.prime(dt)
        for _ in range(5):
            e.advance(dt)
        cycles[mode] = float(np.mean([e.advance(dt).cycles for _ in range(6)]))
        del e
    assert cycles["learned"] < cycles["extrapolate"], cycles
    assert net.status() == 0

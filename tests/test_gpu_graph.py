"""The step as a CUDA graph and the batched ensemble.

With a fixed number of V-cycles the engine's step makes no host read, so it
can be captured once and replayed. Replays must give bit-identical states to
the same steps launched eagerly (same kernels, same order), across re-sorts
that swap the particle buffers. A step split into its solve and push halves is
the whole step, and extra V-cycles between the halves bring a solve that one
cycle left above the tolerance below it; the ensemble's concurrent replays must
advance every run exactly as its own replays do.
"""

from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cluster(n, G, seed):
    rng = np.random.default_rng(seed)
    pos = (rng.normal(size=(n, 3)) * 3.0 + (G - 1) / 2.0).astype(np.float32)
    vel = (rng.normal(size=(n, 3)) * 0.3).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, size=n).astype(np.float32) / n
    return pos, vel, mass


def _engine(G, mode, fixed_cycles=2, tol=1e-6):
    from galaxy_collision_gb300.engine import PMEngine

    e = PMEngine(G, 1.0, tol=tol, sort_every=4, fixed_cycles=fixed_cycles)
    e.set_warmstart(mode, track=True)
    return e


@pytest.mark.parametrize("mode,tol", [("plain", 1e-6), ("extrapolate", 1e-8)])
def test_adaptive_graph_replay_is_bitwise_the_eager_step(cuda, mode, tol):
    """The whole step as one graph with the adaptive solve decided on the device
    (conditional while node): the same V-cycles and bit-identical states as the
    eager steps, which read the residual on the host after every cycle."""
    G, dt = 48, 0.05
    pos, vel, mass = _cluster(50000, G, 3)
    a, b = _engine(G, mode, 0, tol), _engine(G, mode, 0, tol)
    for e in (a, b):
        e.load(pos, vel, mass)
        e.prime(dt)
        for _ in range(3):
            e.advance(dt)
    for _ in range(9):  # crosses two re-sorts (buffer swaps)
        ra = a.advance(dt)
        b.advance_graph(dt)
        rb = b.graph_stats()
        assert rb.cycles == ra.cycles and rb.converged == ra.converged
        assert rb.rel_residual == pytest.approx(ra.rel_residual, rel=1e-12) and rb.rel_residual < tol
    assert len(b._graphs) == 2
    assert any(g.body_launches > 0 for g in b._graphs.values())
    for e in (a, b):
        e.synchronize(dt)
    pa, va, _, _ = a.state_arrays()
    pb, vb, _, _ = b.state_arrays()
    np.testing.assert_array_equal(pa.cpu().numpy(), pb.cpu().numpy())
    np.testing.assert_array_equal(va.cpu().numpy(), vb.cpu().numpy())
    np.testing.assert_array_equal(a.potential().cpu().numpy(), b.potential().cpu().numpy())


@pytest.mark.parametrize("mode", ["plain", "extrapolate"])
def test_graph_replay_is_bitwise_the_eager_step(cuda, mode):
    G, dt = 32, 0.05
    pos, vel, mass = _cluster(40000, G, 1)
    a, b = _engine(G, mode), _engine(G, mode)
    for e in (a, b):
        e.load(pos, vel, mass)
        e.prime(dt)
        for _ in range(3):
            e.advance(dt)
    for _ in range(10):  # crosses two re-sorts (buffer swaps)
        a.advance(dt)
        b.advance_graph(dt)
    assert len(b._graphs) == 2
    for e in (a, b):
        e.synchronize(dt)
    pa, va, _, _ = a.state_arrays()
    pb, vb, _, _ = b.state_arrays()
    np.testing.assert_array_equal(pa.cpu().numpy(), pb.cpu().numpy())
    np.testing.assert_array_equal(va.cpu().numpy(), vb.cpu().numpy())
    assert b.last_residual() < 1e-5


def test_ensemble_steps_every_run_like_its_own_graph(cuda):
    """All runs' step graphs replayed together on their own streams give each run
    exactly the state it gets from its own graph replays one after the other,
    across a re-sort, and every solve meets the tolerance on the device."""
    import torch

    from galaxy_collision_gb300 import ensemble

    a = ensemble.Ensemble(n_runs=3, seed=11, sort_every=3)
    b = ensemble.Ensemble(n_runs=3, seed=11, sort_every=3)
    assert len(a.engines) == 3
    for ens in (a, b):
        ens.prime()
    for _ in range(5):
        a.step()
    for e in b.engines:
        for _ in range(5):
            e.advance_graph(b.dt)
    torch.cuda.synchronize()
    ca = a.counters()
    assert ca["solves"] == 15 and ca["max_rel_residual"] < 1e-6
    for ea, eb in zip(a.engines, b.engines):
        np.testing.assert_array_equal(ea.cur["x"].cpu().numpy(), eb.cur["x"].cpu().numpy())
        np.testing.assert_array_equal(ea.cur["vx"].cpu().numpy(), eb.cur["vx"].cpu().numpy())


def test_autotuned_ensemble_runs_with_the_cached_settings(cuda, tmp_path, monkeypatch):
    """The autotuner times every candidate on a group's first run, caches the
    fastest per (device, grid, count bucket) in JSON, and the ensemble's runs
    step with them; a second ensemble reads the cache without timing again."""
    from galaxy_collision_gb300 import autotune, ensemble

    path = tmp_path / "tune.json"
    monkeypatch.setenv("GC_AUTOTUNE_CACHE", str(path))
    a = ensemble.Ensemble(n_runs=2, seed=11, tuned=True)
    entries = autotune.load(path)
    assert entries and all(set(e["ms_per_step"]) == {autotune._label(c) for c in autotune.CANDIDATES}
                           for e in entries.values())
    for e, st in zip(a.engines, a.settings):
        assert st in [dict(c) for c in autotune.CANDIDATES]
        assert e.sort_every == st["sort_every"]
    monkeypatch.setattr(autotune, "time_candidate", lambda *args, **kw: pytest.fail("re-timed"))
    b = ensemble.Ensemble(n_runs=2, seed=11, tuned=True)
    assert b.settings == a.settings
    a.prime()
    for _ in range(3):
        a.step()
    assert a.counters()["max_rel_residual"] < 1e-6


def test_split_step_is_the_whole_step_and_refine_meets_tol(cuda):
    G, dt = 32, 0.05
    pos, vel, mass = _cluster(30000, G, 2)
    a, b = _engine(G, "plain"), _engine(G, "plain")
    for e in (a, b):
        e.load(pos, vel, mass)
        e.prime(dt)
    for _ in range(3):
        a.advance(dt)
        b.solve_kernels(dt)
        b.push_kernels(dt)
        b.steps_since_sort += 1
    for e in (a, b):
        e.synchronize(dt)
    np.testing.assert_array_equal(a.state_arrays()[0].cpu().numpy(), b.state_arrays()[0].cpu().numpy())
    np.testing.assert_array_equal(a.state_arrays()[1].cpu().numpy(), b.state_arrays()[1].cpu().numpy())

    # one fixed V-cycle from the plain start leaves the solve above 1e-6
    c = _engine(G, "plain")
    c.mg.max_cycles = c.mg.min_cycles = c.fixed_cycles = 1
    c.load(pos, vel, mass)
    c.prime(dt)
    c.solve_kernels(dt)
    import torch

    torch.cuda.synchronize()
    r1 = c.residual_host()
    assert r1 > 1e-6
    extra = c.refine()
    assert extra >= 1
    assert c.last_residual() < 1e-6
    c.push_kernels(dt)
    torch.cuda.synchronize()
    with pytest.raises(Exception):
        c.push_kernels(dt)  # no pending solve


@pytest.mark.parametrize("graph", [False, True])
def test_deposit_next_is_bitwise_the_separate_deposit(cuda, graph):
    """The particle pass that also deposits the drifted positions (GC_STEP_DEPOSIT_NEXT)
    gives the same states and potentials as separate deposit passes, across re-sorts,
    eagerly and replayed from a CUDA graph."""
    import torch

    from galaxy_collision_gb300.engine import PMEngine

    G, dt = 48, 0.05
    pos, vel, mass = _cluster(200_003, G, 4)  # not a multiple of the 1024-particle tile
    mass[::50_000] *= 4000.0  # a few heavy particles take the out-of-line path
    engines = []
    for dn in (False, True):
        e = PMEngine(G, 1.0, tol=1e-6, sort_every=4, fixed_cycles=2 if graph else 0, deposit_next=dn,
                     fixed_point_bits=36)
        e.set_warmstart("extrapolate")
        e.load(pos, vel, mass)
        e.prime(dt)
        for _ in range(3):  # the warm-start history first
            e.advance(dt)
        for _ in range(10):  # crosses two re-sorts
            e.advance_graph(dt) if graph else e.advance(dt)
        engines.append(e)
    a, b = engines
    for k in ("x", "y", "z", "vx", "vy", "vz", "pid"):
        assert torch.equal(a.cur[k], b.cur[k]), k
    pa = torch.empty(G**3, device="cuda")
    pb = torch.empty(G**3, device="cuda")
    a.ctx.call("gc_pm_copy_potential", pa.data_ptr())
    b.ctx.call("gc_pm_copy_potential", pb.data_ptr())
    assert torch.equal(pa, pb)

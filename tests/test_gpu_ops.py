"""GPU parity of the particle<->grid operators against the CPU oracle.

Integer and index work (cell keys, the sort permutation, the fixed-point
density) must be bit-exact; the f32 operators (grad, gather, kick, drift) use
the reference's operation order without contraction on both sides and must be
bit-exact too.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_l2
from oracle import pm

pytestmark = pytest.mark.gpu


def _parts(pos, mass=None, vel=None):
    from galaxy_collision_gb300.data import ParticleState

    pos = np.asarray(pos, np.float32)
    n = pos.shape[0]
    p = ParticleState(n)
    p.pos_x.from_numpy(np.ascontiguousarray(pos[:, 0]))
    p.pos_y.from_numpy(np.ascontiguousarray(pos[:, 1]))
    p.pos_z.from_numpy(np.ascontiguousarray(pos[:, 2]))
    p.mass.from_numpy(np.ones(n, np.float32) if mass is None else np.asarray(mass, np.float32))
    if vel is not None:
        vel = np.asarray(vel, np.float32)
        p.vel_x.from_numpy(np.ascontiguousarray(vel[:, 0]))
        p.vel_y.from_numpy(np.ascontiguousarray(vel[:, 1]))
        p.vel_z.from_numpy(np.ascontiguousarray(vel[:, 2]))
    return p


def _edge_positions(G, dx, rng, n):
    """Random positions plus the edge cases the reference tests touch: on nodes,
    midpoints, the -1 cell, the top cell, just outside, far outside."""
    pos = rng.uniform(-2.0 * dx, (G + 1) * dx, size=(n, 3)).astype(np.float32)
    special = np.array([
        [0.0, 0.0, 0.0], [(G - 1) * dx] * 3, [-0.5 * dx, 1.0, 1.0], [(G - 0.5) * dx, 2.0, 2.0],
        [-dx, 3.0, 3.0], [-1.0001 * dx, 3.0, 3.0], [G * dx, 1.0, 1.0], [1e30, 0.0, 0.0], [-1e30, 0.0, 0.0],
        [8.5 * dx, 8.5 * dx, 8.5 * dx], [np.nextafter(np.float32(G * dx), np.float32(0)), 1.0, 1.0],
    ], dtype=np.float32)
    return np.concatenate([pos, special[:, :3]], axis=0)


@pytest.mark.parametrize("G,dx", [(16, 1.0), (33, 0.375), (64, 2.5)])
def test_cell_keys_bit_exact(cuda, G, dx):
    from galaxy_collision_gb300.deposit import cell_keys

    rng = np.random.default_rng(G)
    pos = _edge_positions(G, dx, rng, 20000)
    keys = cell_keys(_parts(pos), G, dx).cpu().numpy().view(np.uint32)
    np.testing.assert_array_equal(keys, pm.cell_keys(pos, dx, G))


def test_cell_keys_nonfinite_are_sentinel(cuda):
    from galaxy_collision_gb300.deposit import cell_keys

    G = 16
    pos = np.array([[np.nan, 1, 1], [1, np.inf, 1], [1, 1, -np.inf], [2, 2, 2]], np.float32)
    keys = cell_keys(_parts(pos), G, 1.0).cpu().numpy().view(np.uint32)
    assert list(keys[:3]) == [(G + 1) ** 3] * 3
    assert keys[3] == ((3 * 17) + 3) * 17 + 3


@pytest.mark.parametrize("n", [1, 31, 4096, 4097, 100003])
def test_sort_permutation_bit_exact(cuda, n):
    from galaxy_collision_gb300.deposit import sort_keys

    rng = np.random.default_rng(n)
    keys = rng.integers(0, 50, size=n).astype(np.uint32)  # many duplicates: stability matters
    keys[::7] = rng.integers(0, 2**32 - 1, size=keys[::7].shape, dtype=np.uint64).astype(np.uint32)
    kt = torch.from_numpy(keys.view(np.int32)).cuda()
    sk, perm = sort_keys(kt, 16)
    perm = perm.cpu().numpy().view(np.uint32)
    ref = pm.stable_sort_perm(keys)
    np.testing.assert_array_equal(perm, ref)
    np.testing.assert_array_equal(sk.cpu().numpy().view(np.uint32), keys[ref])


@pytest.mark.parametrize("n", [4097, 100003, 1000003])
def test_sort_permutation_nearly_sorted_bit_exact(cuda, n):
    """Nearly sorted keys (the periodic re-sort's case): most warp rounds have
    their digits in lane order and are ranked by runs, the rest by match.any;
    sorted, reversed and constant stretches and the tile tail included."""
    from galaxy_collision_gb300.deposit import sort_keys

    rng = np.random.default_rng(n + 11)
    keys = np.sort(rng.integers(0, max(2, n // 8), size=n)).astype(np.uint32)  # runs of ~8 equal keys
    moved = rng.random(n) < 0.05
    keys[moved] += rng.choice([1, 17, 289, 70000], size=int(moved.sum())).astype(np.uint32)
    q = n // 8
    keys[q:2 * q] = keys[q:2 * q][::-1]  # descending stretch
    keys[2 * q:3 * q] = keys[2 * q]  # one key
    keys[-5:] = np.uint32(0xFFFFFFFF)  # top digits in the last, partial tile
    kt = torch.from_numpy(keys.view(np.int32)).cuda()
    sk, perm = sort_keys(kt, 16)
    ref = pm.stable_sort_perm(keys)
    np.testing.assert_array_equal(perm.cpu().numpy().view(np.uint32), ref)
    np.testing.assert_array_equal(sk.cpu().numpy().view(np.uint32), keys[ref])


def test_pm_resort_of_drifted_particles_at_256(cuda):
    """The engine's re-sort at G = 256 (25-bit cell keys: 9 + 8 + 8 bit passes)
    of particles that left cell order by drifting: the stable permutation."""
    from galaxy_collision_gb300.engine import PMEngine

    G, dx, n = 256, 0.25, 300001
    rng = np.random.default_rng(21)
    cells = np.sort(rng.integers(0, 64 ** 3, size=n))  # a 64^3 block of cells, in cell order
    ijk = np.stack([cells // 4096, (cells // 64) % 64, cells % 64], axis=1) + 96
    pos = ((ijk + rng.uniform(0.0, 1.0, size=(n, 3))) * dx).astype(np.float32)
    pos += rng.normal(scale=0.15 * dx, size=pos.shape).astype(np.float32)  # drift
    pos[:3] = [[-5.0, 1.0, 1.0], [np.nan, 2.0, 2.0], [30.0, 30.0, 70.0]]  # outside / non-finite / face
    vel = np.zeros_like(pos)
    mass = np.ones(n, np.float32)
    eng = PMEngine(G, dx, sort_every=0)
    eng.load(pos, vel, mass, None, sort=False)
    eng.sort()
    perm = pm.stable_sort_perm(pm.cell_keys(pos, dx, G))
    cur = {k: v.cpu().numpy() for k, v in eng.cur.items() if not k.startswith("_")}
    np.testing.assert_array_equal(cur["pid"], perm.astype(np.int32))
    np.testing.assert_array_equal(cur["z"], pos[perm, 2])


def test_pm_sort_permutes_all_arrays(cuda):
    from galaxy_collision_gb300.engine import PMEngine

    G, dx, n = 32, 1.0, 30001
    rng = np.random.default_rng(7)
    pos = rng.uniform(-1, G, size=(n, 3)).astype(np.float32)
    vel = rng.normal(size=(n, 3)).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, size=n).astype(np.float32)
    gid = rng.integers(0, 2, size=n).astype(np.int32)
    eng = PMEngine(G, dx, sort_every=0)
    eng.load(pos, vel, mass, gid, sort=True)
    perm = pm.stable_sort_perm(pm.cell_keys(pos, dx, G))
    cur = {k: v.cpu().numpy() for k, v in eng.cur.items() if not k.startswith("_")}
    np.testing.assert_array_equal(cur["pid"], perm.astype(np.int32))
    np.testing.assert_array_equal(cur["x"], pos[perm, 0])
    np.testing.assert_array_equal(cur["vz"], vel[perm, 2])
    np.testing.assert_array_equal(cur["m"], mass[perm])
    np.testing.assert_array_equal(cur["gid"], gid[perm])


def test_pm_sort_ahead_orders_by_predicted_cells(cuda):
    """gc_pm_sort_ahead: keys of x + v*tau (f32, rounded per operation), the
    current cell where the predicted position deposits nothing; stable."""
    from galaxy_collision_gb300.engine import PMEngine

    G, dx, n, dt = 32, 1.0, 30001, 0.1
    rng = np.random.default_rng(8)
    pos = rng.uniform(-1, G, size=(n, 3)).astype(np.float32)
    vel = rng.normal(scale=4.0, size=(n, 3)).astype(np.float32)
    vel[:5] = [[np.nan, 0, 0], [np.inf, 0, 0], [0, -np.inf, 0], [1e30, 0, 0], [0, 0, -40.0]]
    mass = rng.uniform(0.5, 1.5, size=n).astype(np.float32)
    eng = PMEngine(G, dx, sort_every=0, sort_ahead=5.0)
    eng.load(pos, vel, mass, None, sort=False)
    eng.sort(dt)
    tau = np.float32(5.0 * dt)
    with np.errstate(invalid="ignore", over="ignore"):
        ahead = pos + vel * tau
    k_ahead, k_now = pm.cell_keys(ahead, dx, G), pm.cell_keys(pos, dx, G)
    keys = np.where(k_ahead != (G + 1) ** 3, k_ahead, k_now)
    assert (keys != k_now).mean() > 0.5
    perm = pm.stable_sort_perm(keys)
    cur = {k: v.cpu().numpy() for k, v in eng.cur.items() if not k.startswith("_")}
    np.testing.assert_array_equal(cur["pid"], perm.astype(np.int32))
    np.testing.assert_array_equal(cur["y"], pos[perm, 1])
    np.testing.assert_array_equal(cur["vx"], vel[perm, 0])
    # tau = 0 is the plain cell sort
    eng0 = PMEngine(G, dx, sort_every=0)
    eng0.load(pos, vel, mass, None, sort=False)
    eng0.sort(dt)
    np.testing.assert_array_equal(eng0.cur["pid"].cpu().numpy(), pm.stable_sort_perm(k_now).astype(np.int32))


@pytest.mark.parametrize("G,dx,bits", [(16, 1.0, 52), (48, 0.375, 52), (64, 2.5, 40), (33, 1.0, 56)])
def test_deposit_bit_exact_vs_fixed_point_oracle(cuda, G, dx, bits):
    from galaxy_collision_gb300.data import Field
    from galaxy_collision_gb300.deposit import deposit_density

    rng = np.random.default_rng(G + bits)
    pos = _edge_positions(G, dx, rng, 50000)
    mass = rng.uniform(0.1, 3.0, size=pos.shape[0]).astype(np.float32)
    rho = Field((G, G, G))
    deposit_density(_parts(pos, mass), rho, dx, fixed_point_bits=bits)
    ref, _, _ = pm.deposit_fixed(pos, mass, dx, G, bits)
    np.testing.assert_array_equal(rho.to_numpy(), ref)


@pytest.mark.parametrize("dx,offset", [(0.25, 0), (0.25, 1), (0.375, 0), (0.375, 3)])
def test_deposit_dense_sorted_runs_bit_exact(cuda, dx, offset):
    """Cell-sorted particles packed into a dozen cells (long runs merged across
    the warp), a few heavy particles (contributions above 2^22 quanta, the
    general conversion), edge cells, and array starts that are not 16-byte
    aligned (scalar loads). dx = 0.25 takes the exact reciprocal multiply."""
    from types import SimpleNamespace

    from galaxy_collision_gb300.data import Field
    from galaxy_collision_gb300.deposit import deposit_density

    G, bits, n = 32, 40, 70001
    rng = np.random.default_rng(int(dx * 1000) + offset)
    cells = rng.integers(-1, G, size=(12, 3))
    pick = rng.integers(0, 12, size=n)
    pos = ((cells[pick] + rng.uniform(0.0, 1.0, size=(n, 3))) * dx).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, size=n).astype(np.float32)
    mass[rng.integers(0, n, size=20)] = 5.0e4
    order = pm.stable_sort_perm(pm.cell_keys(pos, dx, G))
    pos, mass = pos[order], mass[order]

    def dev(a):
        t = torch.zeros(n + offset, dtype=torch.float32, device="cuda")
        t[offset:] = torch.from_numpy(np.ascontiguousarray(a)).cuda()
        return t[offset:]

    parts = SimpleNamespace(n=n, pos_x=dev(pos[:, 0]), pos_y=dev(pos[:, 1]), pos_z=dev(pos[:, 2]), mass=dev(mass))
    rho = Field((G, G, G))
    deposit_density(parts, rho, dx, fixed_point_bits=bits)
    ref, _, _ = pm.deposit_fixed(pos, mass, dx, G, bits)
    np.testing.assert_array_equal(rho.to_numpy(), ref)


def test_deposit_vs_fp64_oracle(cuda):
    from galaxy_collision_gb300.data import Field
    from galaxy_collision_gb300.deposit import deposit_density

    G, dx = 64, 0.375
    rng = np.random.default_rng(11)
    pos = (rng.normal(size=(200000, 3)) * 3.0 + 12.0).astype(np.float32)
    mass = np.full(pos.shape[0], 1.0 / pos.shape[0], np.float32)
    rho = Field((G, G, G))
    deposit_density(_parts(pos, mass), rho, dx)
    ref = pm.deposit_f64(pos, mass, dx, G)
    assert rel_l2(rho.to_numpy(), ref) <= 1e-6
    # mass conservation for the in-box particles
    assert rho.to_numpy().astype(np.float64).sum() * dx**3 == pytest.approx(ref.sum() * dx**3, rel=1e-9)


def test_deposit_reference_known_answers(cuda):  # tests/test_deposit.py:76-162
    from galaxy_collision_gb300.data import GridState
    from galaxy_collision_gb300.deposit import deposit_density

    dx = 2.5
    g = GridState(8)
    deposit_density(_parts([[2 * dx, 3 * dx, 4 * dx]], [5.0]), g.rho, dx)
    rho = g.rho.to_numpy()
    assert rho[2, 3, 4] == pytest.approx(5.0 / dx**3) and rho.sum() == pytest.approx(5.0 / dx**3)
    g = GridState(16)
    deposit_density(_parts([[8.5, 8.5, 8.5]], [8.0]), g.rho, 1.0)
    assert np.allclose(g.rho.to_numpy()[8:10, 8:10, 8:10], 1.0)
    deposit_density(_parts([[-3.0, 8, 8], [40.0, 8, 8], [15.5, 8, 8]], [1, 1, 1]), g.rho, 1.0)
    rho = g.rho.to_numpy()
    assert rho.sum() <= 3.0 + 1e-5 and rho[15, 8, 8] == pytest.approx(0.5) and rho[0].sum() == 0.0


def test_deposit_order_independent_and_reproducible(cuda):
    from galaxy_collision_gb300.data import Field
    from galaxy_collision_gb300.deposit import deposit_density

    G = 32
    rng = np.random.default_rng(3)
    pos = (rng.normal(size=(300000, 3)) * 1.5 + 15.0).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, size=pos.shape[0]).astype(np.float32)
    out = []
    for order in (np.arange(pos.shape[0]), rng.permutation(pos.shape[0]), np.argsort(pos[:, 0])):
        rho = Field((G, G, G))
        deposit_density(_parts(pos[order], mass[order]), rho, 1.0)
        out.append(rho.to_numpy())
    np.testing.assert_array_equal(out[0], out[1])
    np.testing.assert_array_equal(out[0], out[2])


def test_fixed_point_bits_limit_is_enforced(cuda):
    from galaxy_collision_gb300.data import Field
    from galaxy_collision_gb300.deposit import deposit_density

    G = 33  # (G-1) * 2^bits must stay below 2^62 for the exact moment sums: bits <= 56
    with pytest.raises(ValueError, match="fixed_point_bits"):
        deposit_density(_parts([[4.0, 4.0, 4.0]], [1.0]), Field((G, G, G)), 1.0, fixed_point_bits=57)


def test_nonfinite_position_flagged_and_skipped(cuda):
    from galaxy_collision_gb300._ops import op_context
    from galaxy_collision_gb300.data import Field
    from galaxy_collision_gb300.deposit import deposit_density

    G = 16
    op_context(G, 1.0).status(clear=True)
    rho = Field((G, G, G))
    deposit_density(_parts([[np.nan, 4, 4], [4.0, 4.0, 4.0]], [1.0, 2.0]), rho, 1.0)
    assert op_context(G, 1.0).status(clear=True) & 0x1
    r = rho.to_numpy()
    assert r[4, 4, 4] == pytest.approx(2.0) and r.sum() == pytest.approx(2.0)


@pytest.mark.parametrize("G,dx", [(16, 1.0), (40, 0.375)])
def test_grad_bit_exact(cuda, G, dx):
    from galaxy_collision_gb300.data import Field, GridState
    from galaxy_collision_gb300.deposit import potential_to_accel

    rng = np.random.default_rng(G)
    phi = rng.normal(size=(G, G, G)).astype(np.float32)
    g = GridState(G)
    g.phi.from_numpy(phi)
    potential_to_accel(g.phi, g.ax, g.ay, g.az, dx)
    ref = pm.grad(phi, dx)
    for a, b in zip((g.ax, g.ay, g.az), ref):
        np.testing.assert_array_equal(a.to_numpy(), b)
    assert isinstance(g.ax, Field)


def test_gather_bit_exact(cuda):
    from galaxy_collision_gb300.data import Field, GridState
    from galaxy_collision_gb300.deposit import gather_acceleration

    G, dx = 24, 0.5
    rng = np.random.default_rng(9)
    pos = _edge_positions(G, dx, rng, 30000)
    grids = [rng.normal(size=(G, G, G)).astype(np.float32) for _ in range(3)]
    g = GridState(G)
    for f, a in zip((g.ax, g.ay, g.az), grids):
        f.from_numpy(a)
    n = pos.shape[0]
    acc = [Field(n) for _ in range(3)]
    gather_acceleration(_parts(pos), g.ax, g.ay, g.az, *acc, dx)
    ref = pm.gather(pos, *grids, dx)
    for a, b in zip(acc, ref):
        np.testing.assert_array_equal(a.to_numpy(), b)


def test_kick_drift_bit_exact(cuda):
    from galaxy_collision_gb300.data import Field
    from galaxy_collision_gb300.integrator import drift, kick

    n = 10007
    rng = np.random.default_rng(1)
    arrs = [rng.normal(size=n).astype(np.float32) for _ in range(9)]
    f = [Field(n) for _ in range(9)]
    for fi, a in zip(f, arrs):
        fi.from_numpy(a)
    kick(*f[3:6], *f[6:9], n, 0.013)
    drift(*f[0:3], *f[3:6], n, 0.026)
    ref = [a.copy() for a in arrs]
    pm.axpy3(*ref[3:6], *ref[6:9], np.float32(0.013))
    pm.axpy3(*ref[0:3], *ref[3:6], np.float32(0.026))
    for fi, r in zip(f[:6], ref[:6]):
        np.testing.assert_array_equal(fi.to_numpy(), r)


def test_kdk_step_bit_identical_to_inline_loop(cuda):  # tests/test_integrator.py:189-257
    from galaxy_collision_gb300.data import Field, GridState
    from galaxy_collision_gb300.deposit import deposit_density, gather_acceleration, potential_to_accel
    from galaxy_collision_gb300.integrator import drift, kdk_step, kick
    from galaxy_collision_gb300.solver import make_solver

    G, n, dt = 32, 2000, 0.05
    rng = np.random.default_rng(2)
    pos = (rng.normal(size=(n, 3)) * 2.0 + 15.5).astype(np.float32)
    vel = (rng.normal(size=(n, 3)) * 0.2).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)

    def chain(parts):
        grid = GridState(G)
        acc = [Field(n) for _ in range(3)]
        solver = make_solver("multigrid", G, grav_constant=1.0, tol=1e-6, n_cycles=30)

        def accel_fn():
            deposit_density(parts, grid.rho, 1.0)
            solver.solve(grid.rho, grid.phi, warm_start=False)
            potential_to_accel(grid.phi, grid.ax, grid.ay, grid.az, 1.0)
            gather_acceleration(parts, grid.ax, grid.ay, grid.az, *acc, 1.0)

        return acc, accel_fn

    p1 = _parts(pos, mass, vel)
    acc1, f1 = chain(p1)
    calls = {"n": 0}

    def counted():
        calls["n"] += 1
        f1()

    counted()
    for _ in range(5):
        kdk_step(p1, *acc1, counted, dt)
    assert calls["n"] == 6
    p2 = _parts(pos, mass, vel)
    acc2, f2 = chain(p2)
    for _ in range(5):
        f2()
        kick(p2.vel_x, p2.vel_y, p2.vel_z, *acc2, n, dt / 2)
        drift(p2.pos_x, p2.pos_y, p2.pos_z, p2.vel_x, p2.vel_y, p2.vel_z, n, dt)
        f2()
        kick(p2.vel_x, p2.vel_y, p2.vel_z, *acc2, n, dt / 2)
    for a, b in zip(p1.fields()[:6], p2.fields()[:6]):
        np.testing.assert_array_equal(a.to_numpy(), b.to_numpy())


def test_import_export_round_trip(cuda):
    """gc_pm_import splits the reference's N x 3 layout into the engine's arrays
    (origin subtracted in f64); gc_pm_export writes them back in the original
    order after sorts and steps, equal to state_arrays."""
    import ctypes as C

    from galaxy_collision_gb300.engine import PMEngine

    G, dx = 32, 0.5
    origin = (-8.0, -8.0, -8.0)
    rng = np.random.default_rng(12)
    n = 20011
    pos = rng.uniform(-7.0, 7.0, size=(n, 3)).astype(np.float32)
    vel = rng.normal(size=(n, 3)).astype(np.float32)
    mass = rng.uniform(0.5, 1.5, size=n).astype(np.float32) / n
    gid = rng.integers(0, 3, size=n).astype(np.int32)
    eng = PMEngine(G, dx, origin=origin, sort_every=3)
    eng.load(pos, vel, mass, gid, sort=True)
    rel = (pos.astype(np.float64) - np.asarray(origin)).astype(np.float32)
    cur = {k: eng.cur[k].cpu().numpy() for k in ("x", "y", "z", "vx", "m", "gid", "pid")}
    pid = cur["pid"]
    np.testing.assert_array_equal(np.sort(pid), np.arange(n))
    np.testing.assert_array_equal(cur["x"], rel[pid, 0])
    np.testing.assert_array_equal(cur["z"], rel[pid, 2])
    np.testing.assert_array_equal(cur["vx"], vel[pid, 0])
    np.testing.assert_array_equal(cur["m"], mass[pid])
    np.testing.assert_array_equal(cur["gid"], gid[pid])
    # the sorted import equals import + sort
    e2 = PMEngine(G, dx, origin=origin, sort_every=3)
    e2.load(pos, vel, mass, gid, sort=False)
    np.testing.assert_array_equal(e2.cur["pid"].cpu().numpy(), np.arange(n, dtype=np.int32))
    e2.sort()
    for k in ("x", "y", "z", "vx", "vy", "vz", "m", "gid", "pid"):
        np.testing.assert_array_equal(e2.cur[k].cpu().numpy(), eng.cur[k].cpu().numpy())
    # pinned host arrays (each gathered as its copy lands), no gid: gid zeros
    e3 = PMEngine(G, dx, origin=origin, sort_every=3)
    e3.cur = e3._alloc(n)
    e3.cur["gid"].fill_(7)
    e3.alt = e3._alloc(n)
    e3.load(torch.from_numpy(pos).pin_memory(), torch.from_numpy(vel).pin_memory(),
            torch.from_numpy(mass).pin_memory(), None, sort=True)
    for k in ("x", "y", "z", "vx", "vy", "vz", "m", "pid"):
        np.testing.assert_array_equal(e3.cur[k].cpu().numpy(), eng.cur[k].cpu().numpy())
    assert not e3.cur["gid"].any()
    # the kept order serves gathers of any subset, in any order, until the next sort
    o = e3._struct(e3.alt)
    posd, veld, md = (torch.from_numpy(a).cuda() for a in (pos, vel, mass))
    oc = e3._origin_c()
    e3.ctx.call("gc_pm_import_order", posd.data_ptr(), oc, n, what="order")
    e3.ctx.call("gc_pm_import_gather", None, None, md.data_ptr(), None, oc, C.byref(o), what="gather m")
    e3.ctx.call("gc_pm_import_gather", None, veld.data_ptr(), None, None, oc, C.byref(o), what="gather vel")
    e3.ctx.call("gc_pm_import_gather", posd.data_ptr(), None, None, None, oc, C.byref(o), what="gather pos")
    for k in ("x", "y", "z", "vx", "vy", "vz", "m", "pid"):
        np.testing.assert_array_equal(e3.alt[k].cpu().numpy(), eng.cur[k].cpu().numpy())
    e3.sort()  # the sort reuses the scratch: the kept order is gone
    with pytest.raises(Exception, match="gc_pm_import_order"):
        e3.ctx.call("gc_pm_import_gather", posd.data_ptr(), None, None, None, oc, C.byref(o), what="gather pos")
    p, v, m, g = eng.export()
    back = (rel.astype(np.float64) + np.asarray(origin)).astype(np.float32)
    np.testing.assert_array_equal(p.numpy(), back)
    np.testing.assert_array_equal(v.numpy(), vel)
    np.testing.assert_array_equal(m.numpy(), mass)
    np.testing.assert_array_equal(g.numpy(), gid)
    eng.prime(0.01)
    for _ in range(7):  # crosses two re-sorts
        eng.advance(0.01)
    eng.synchronize(0.01)
    pp = torch.empty((n, 3), dtype=torch.float32).pin_memory()
    vd = torch.empty((n, 3), dtype=torch.float32, device="cuda")
    eng.export(pp, vd)
    torch.cuda.synchronize()
    ps, vs, _, _ = eng.state_arrays(physical=True)
    np.testing.assert_array_equal(pp.numpy(), ps.to(torch.float32).cpu().numpy())
    np.testing.assert_array_equal(vd.cpu().numpy(), vs.cpu().numpy())
    # many overlapped ranges (pinned and pageable host outputs) == gc_pm_export's scatter
    eng._export_ranges = lambda k: PMEngine._export_ranges(k, per=3000)
    assert len(eng._export_ranges(n)) == 7
    pp2 = torch.zeros((n, 3), dtype=torch.float32).pin_memory()
    mm2, gg2 = torch.zeros(n, dtype=torch.float32), torch.zeros(n, dtype=torch.int32).pin_memory()
    eng.export(pp2, None, mm2, gg2)
    torch.cuda.synchronize()
    ref = [torch.zeros((n, 3), dtype=torch.float32, device="cuda"), torch.zeros(n, dtype=torch.float32, device="cuda"),
           torch.zeros(n, dtype=torch.int32, device="cuda")]
    eng.ctx.call("gc_pm_export", C.byref(eng._struct(eng.cur)), eng._origin_c(), ref[0].data_ptr(), None,
                 ref[1].data_ptr(), ref[2].data_ptr(), what="gc_pm_export")
    np.testing.assert_array_equal(pp2.numpy(), ref[0].cpu().numpy())
    np.testing.assert_array_equal(mm2.numpy(), ref[1].cpu().numpy())
    np.testing.assert_array_equal(gg2.numpy(), ref[2].cpu().numpy())
    np.testing.assert_array_equal(gg2.numpy(), gid)
    with pytest.raises(Exception, match=r"range \[0, 20012\) outside"):
        eng.ctx.call("gc_pm_export_range", C.byref(eng._struct(eng.cur)), eng._origin_c(), ref[0].data_ptr(), None,
                     None, None, 0, n + 1, what="gc_pm_export_range")
    assert eng.ctx.status() & 0x4 == 0
    # ranks made for one particle set are refused for another of the same size
    eng.ctx.call("gc_pm_export_order", C.byref(eng._struct(eng.cur)), what="gc_pm_export_order")
    with pytest.raises(Exception, match=r"another particle set"):
        eng.ctx.call("gc_pm_export_range", C.byref(eng._struct(eng.alt)), eng._origin_c(), ref[0].data_ptr(), None,
                     None, None, 0, n, what="gc_pm_export_range")
    # a pid outside [0, n): flagged at the inversion, its original index left untouched and flagged
    q = int(eng.cur["pid"][0])
    eng.cur["pid"][0] = -1
    out = torch.full((n,), -5.0, dtype=torch.float32, device="cuda")
    src = eng._struct(eng.cur)
    eng.ctx.call("gc_pm_export_order", C.byref(src), what="gc_pm_export_order")
    eng.ctx.call("gc_pm_export_range", C.byref(src), eng._origin_c(), None, None, out.data_ptr(), None, 0, n,
                 what="gc_pm_export_range")
    assert eng.ctx.status(clear=True) & 0x4
    o = out.cpu().numpy()
    assert o[q] == -5.0
    np.testing.assert_array_equal(np.delete(o, q), np.delete(mass, q))

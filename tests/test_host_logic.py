"""Host-side logic without a GPU: configuration, snapshot layout, initial
conditions, benchmark bookkeeping and the multi-process replica aggregation."""

from __future__ import annotations

import json
import multiprocessing as mp
import os
import socket

import numpy as np
import pytest

from conftest import ROOT


# ---- config (reference config.py:35-147) -------------------------------------
def test_config_defaults_and_validation():
    from galaxy_collision_gb300.config import ConfigError, SimConfig

    c = SimConfig()
    assert (c.grid_size, c.solver, c.dt, c.steps) == (256, "multigrid", 0.01, 1)
    with pytest.raises(ConfigError, match="only one resolution knob"):
        SimConfig(n_particles=10, particle_mass=1.0)
    with pytest.raises(ConfigError, match="solver"):
        SimConfig(solver="spectral")
    with pytest.raises(ConfigError, match="dt"):
        SimConfig(dt=0.0)
    assert SimConfig(particle_mass=2.32e11).resolve_n_particles() == 2
    assert isinstance(ConfigError("x"), ValueError)


def test_flat_yaml_loader(tmp_path):
    from galaxy_collision_gb300.config import ConfigError, dump_config, from_dict, load_config, parse_flat_yaml

    text = """# a comment
name: paper-4v
backend: cuda
ic_preset: two_disk      # inline comment
grid_size: 256
n_particles: 10000000
dt: 0.5
grav_constant: null
output_dir: 'outputs/run # 1'
seed: 0
"""
    d = parse_flat_yaml(text)
    assert d == {"name": "paper-4v", "backend": "cuda", "ic_preset": "two_disk", "grid_size": 256,
                 "n_particles": 10000000, "dt": 0.5, "grav_constant": None, "output_dir": "outputs/run # 1",
                 "seed": 0}
    p = tmp_path / "c.yaml"
    p.write_text(text)
    c = load_config(p)
    assert c.n_particles == 10_000_000 and c.output_dir == "outputs/run # 1"
    dump_config(c, tmp_path / "d.yaml")
    assert load_config(tmp_path / "d.yaml") == c
    with pytest.raises(ConfigError, match="unknown config keys"):
        from_dict({"name": "x", "bogus": 1})
    with pytest.raises(ConfigError, match="flat"):
        parse_flat_yaml("a:\n  b: 1\n")
    with pytest.raises(ConfigError, match="not found"):
        load_config(tmp_path / "missing.yaml")


def test_repo_configs_load():
    from galaxy_collision_gb300.config import load_config

    files = sorted((ROOT / "configs").glob("*.yaml"))
    assert files
    for f in files:
        load_config(f)


# ---- snapshots (reference io.py) ----------------------------------------------
def test_snapshot_npz_roundtrip(tmp_path):
    from galaxy_collision_gb300.io import Snapshot, read_snapshot, write_snapshot

    rng = np.random.default_rng(0)
    s = Snapshot(step=7, time=3.5, pos=rng.normal(size=(100, 3)).astype(np.float32),
                 vel=rng.normal(size=(100, 3)).astype(np.float32), mass=np.ones(100, np.float32),
                 gid=np.arange(100, dtype=np.int32) % 2, dx=0.25, rho=rng.random((8, 8, 8)).astype(np.float32),
                 phi=None, diagnostics={"energy": np.float64(-1.5), "momentum": np.array([1.0, 2.0, 3.0])})
    p = write_snapshot(s, tmp_path / "snap.npz")
    r = read_snapshot(p)
    assert (r.step, r.time, r.dx) == (7, 3.5, 0.25)
    np.testing.assert_array_equal(r.pos, s.pos)
    np.testing.assert_array_equal(r.gid, s.gid)
    np.testing.assert_array_equal(r.rho, s.rho)
    assert r.phi is None
    assert float(r.diagnostics["energy"]) == -1.5
    np.testing.assert_array_equal(r.diagnostics["momentum"], [1.0, 2.0, 3.0])
    with np.load(p) as z:  # the reference's key layout (io.py:160-174)
        assert {"step", "time", "dx", "pos", "vel", "mass", "gid", "rho", "diag__energy"} <= set(z.files)
    with pytest.raises(ValueError, match="extension"):
        write_snapshot(s, tmp_path / "snap.txt")
    with pytest.raises(FileNotFoundError):
        read_snapshot(tmp_path / "none.npz")


# ---- initial conditions ---------------------------------------------------------
def test_plummer_sampler_properties():
    from galaxy_collision_gb300 import ic
    from oracle import diagnostics as odiag

    p = ic.plummer(131072, seed=0)
    r = np.linalg.norm(p.pos.astype(np.float64), axis=1)
    assert p.n == 131072 and r.max() <= 10.0 + 1e-5
    assert p.mass.astype(np.float64).sum() == pytest.approx(1.0, rel=1e-6)
    # half-mass radius of a Plummer sphere truncated at 10a: ~1.30a (untruncated 1.305a)
    assert np.median(r) == pytest.approx(1.30, rel=0.03)
    sub = slice(0, 3000)
    m = p.mass.astype(np.float64)[sub] * (131072 / 3000)
    ke = odiag.kinetic_energy(m, p.vel[sub])
    pe = odiag.potential_energy_direct(m, p.pos[sub], softening=0.02)
    assert odiag.virial_ratio(ke, pe) == pytest.approx(0.5, abs=0.08)
    assert np.array_equal(ic.plummer(1000, seed=3).pos, ic.plummer(1000, seed=3).pos)


def test_two_disk_sampler_properties():
    from galaxy_collision_gb300 import ic

    d = ic.two_disk(20000, 30000, seed=1)
    assert d.n == 50000
    m = d.mass.astype(np.float64)
    assert m[d.gid == 0].sum() == pytest.approx(1.01, rel=1e-5)  # disk 1.0 + 1% central mass
    assert m[d.gid == 1].sum() == pytest.approx(1.515, rel=1e-5)
    cm = (m[:, None] * d.pos).sum(0) / m.sum()
    assert np.abs(cm).max() < 0.05
    p = (m[:, None] * d.vel).sum(0)
    assert np.abs(p).max() < 0.01
    g1 = d.gid == 1
    c1 = (m[g1, None] * d.pos[g1]).sum(0) / m[g1].sum()
    c0 = (m[~g1, None] * d.pos[~g1]).sum(0) / m[~g1].sum()
    np.testing.assert_allclose(c1 - c0, [20.0, 2.0, 0.0], atol=0.1)
    # disk 2 inclined 30 deg about x: its angular momentum is tilted from z by 30 deg
    L = (m[g1, None] * np.cross(d.pos[g1] - c1, d.vel[g1])).sum(0)
    tilt = np.degrees(np.arccos(L[2] / np.linalg.norm(L)))
    assert tilt == pytest.approx(30.0, abs=1.5)


# ---- engine host logic -------------------------------------------------------
@pytest.mark.parametrize("n,per", [(1, 8), (7, 8), (8, 8), (9, 8), (100_000_000, 1 << 23), (20011, 3000)])
def test_export_ranges_partition(n, per):
    """The overlapped export's ranges tile [0, n) in order, at most `per` each."""
    from galaxy_collision_gb300.engine import PMEngine

    r = PMEngine._export_ranges(n, per=per)
    assert r[0][0] == 0 and r[-1][1] == n
    assert all(a[1] == b[0] for a, b in zip(r[:-1], r[1:]))
    assert all(0 < q1 - q0 <= per for q0, q1 in r)
    assert len(r) == -(-n // per)


# ---- benchmark bookkeeping ----------------------------------------------------
def test_bench_roofline_and_traffic_parse(tmp_path):
    import bench

    stats = {"gather_kick_drift": (10, 10, 20.0), "smooth0": (400, 400, 30.0), "reduce": (50, 50, 1.0)}
    r = bench._roofline(stats, n=1_000_000, G=128, hbm_gbs=6783.1, traffic={"smooth0": 12.0})
    assert r["kernel"] == "smooth0"
    per_launch = bench.ALGO_BYTES["smooth0"][1] * 128**3
    assert r["achieved"] == pytest.approx(per_launch / (30.0 / 400 / 1e3) / 1e9, rel=1e-3)
    assert r["frac"] == pytest.approx(r["achieved"] / 6783.1, abs=1e-4)
    assert r["traffic"] == 12.0 * 128**3


def test_bench_clock_sampler_parse(tmp_path):
    import bench

    cs = bench.ClockSampler(0)
    cs.path = str(tmp_path / "c.csv")
    (tmp_path / "c.csv").write_text("0, 1965, 2070, 900.1, 0x0, Not Active, Not Active, Not Active, Not Active\n"
                                    "0, 1995, 2070, 950.2, 0x4, Not Active, Not Active, Not Active, Active\n")

    class P:
        def terminate(self):
            pass

        def wait(self, timeout=None):
            return 0

    cs.proc = P()
    out = cs.stop()
    assert out["sm_mhz"] == 1980.0 and out["sm_max_mhz"] == 2070.0 and out["reasons"] == ["sw_power_cap"]


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _replica_worker(rank, world, port, ms, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    q.put((rank, bench.aggregate(ms[rank], 1000 * (rank + 1), 5, world)))
    dist.destroy_process_group()


def test_replica_aggregation_gloo_two_ranks():
    """Replicas only: the step has no collective; the bench reduces the slowest
    rank's time and the particles of all ranks."""
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ms = [100.0, 250.0]
    procs = [ctx.Process(target=_replica_worker, args=(r, 2, port, ms, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        ms_max, value = out[r]
        assert ms_max == 250.0
        assert value == pytest.approx(3000 * 5 / 0.25)


def test_bench_json_contract_keys():
    """The reference arm's line carries the keys the driver reads."""
    import subprocess
    import sys

    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--config", "plummer_131k",
                        "--scale", "0.05", "--steps", "2", "--warmup", "1"], capture_output=True, text=True,
                       timeout=300, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in line
    assert line["impl"] == "reference" and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["value"] > 0

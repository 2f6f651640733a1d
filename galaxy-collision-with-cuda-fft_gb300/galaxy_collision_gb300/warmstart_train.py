"""Training data, training loop and evaluation of the learned warm start.

Training pairs come from the multigrid itself: randomised two-disk collisions
(mass ratio U[1,3], impact parameter U[0,5], inclination U[0,90] degrees,
approach speed U[0.2,1.0]) advance in the fused engine with the plain warm
start; every ``every`` steps the engine records the network's input features
and the second difference of the potential its converged solve produced (f16,
(G/2)^3). The
network (``WarmStartNet``) is trained on them with its own tensor-core
forward/backward kernels and Adam. Evaluation runs held-out collisions with the
plain, extrapolated and learned initial guesses and reports V-cycles and solve
time to the same relative residual.

Command line (writes the package's weight file)::

    python -m galaxy_collision_gb300.warmstart_train --runs 200 --steps 100 --every 10 --epochs 20
"""

from __future__ import annotations

import argparse
import time
from pathlib import Path

import numpy as np
import torch

from galaxy_collision_gb300 import ic
from galaxy_collision_gb300.engine import PMEngine
from galaxy_collision_gb300.warmstart import WEIGHTS_PATH, WarmStartNet

BOX, GRID, DT = 64.0, 256, 0.005

# kernels of one solve: the multigrid, its faces, norms and b0 conversion, and the initial guess
SOLVE_KERNELS = ("smooth0", "update0", "resid0", "resid0e", "restrict", "smooth", "resid", "prolong", "prolong0",
                 "coarse", "tail", "faces", "moments", "rhs", "reduce", "convert_q", "warmstart")


def random_collision(rng: np.random.Generator, n: int, dx: float = BOX / GRID) -> ic.ICResult:
    ratio = rng.uniform(1.0, 3.0)
    b = rng.uniform(0.0, 5.0)
    inc = rng.uniform(0.0, 90.0)
    v = rng.uniform(0.2, 1.0)
    n1 = max(2, int(round(n / (1.0 + ratio))))
    return ic.two_disk(n1, max(2, n - n1), seed=int(rng.integers(1 << 31)), m1=1.0, m2=ratio, incline_deg=inc,
                       separation=(20.0, b, 0.0), approach_speed=v, dx=dx)


def _engine(grid: int, box: float, tol: float) -> PMEngine:
    return PMEngine(grid, box / grid, grav=1.0, origin=(-box / 2.0,) * 3, tol=tol, max_cycles=60, sort_every=20,
                    fixed_point_bits=40)


def generate_samples(n_runs: int, n_particles: int = 1_000_000, steps: int = 100, every: int = 10, seed: int = 0,
                     grid: int = GRID, box: float = BOX, dt: float = DT, tol: float = 1e-6, log=None) -> torch.Tensor:
    """(S, 5, R, R, R) float16 on the device: channels 0..3 features, 4 target."""
    R = grid // 2
    rng = np.random.default_rng(seed)
    per_run = len([s for s in range(1, steps + 1) if s % every == 0 and s >= 4])
    out = torch.empty((n_runs * per_run, 5, R, R, R), dtype=torch.float16, device="cuda")
    k = 0
    for run in range(n_runs):
        t0 = time.time()
        icr = random_collision(rng, n_particles, box / grid)
        eng = _engine(grid, box, tol)
        eng.set_warmstart("plain", track=True)
        eng.load(icr.pos, icr.vel, icr.mass, icr.gid)
        eng.prime(dt)
        for s in range(1, steps + 1):
            if s % every == 0 and s >= 4:
                eng.record_sample(out[k])
                k += 1
            eng.advance(dt)
        torch.cuda.synchronize()
        if log:
            log(f"run {run + 1}/{n_runs}: {k} samples, {time.time() - t0:.1f}s")
        del eng
    return out[:k]


def train(net: WarmStartNet, samples: torch.Tensor, epochs: int = 20, lr: float = 1e-3, seed: int = 0,
          log=None) -> list[float]:
    """Adam over the samples, one sample per step, reshuffled every epoch. Returns
    the mean loss of each epoch."""
    rng = np.random.default_rng(seed)
    S = samples.shape[0]
    hist = []
    for ep in range(epochs):
        acc = torch.zeros(1, dtype=torch.float64, device=samples.device)
        t0 = time.time()
        for i in rng.permutation(S):
            net.forward(samples[i, :4])
            acc += net.backward(samples[i, 4]).double()
            net.adam_step(lr)
        hist.append(float(acc.item()) / S)
        if net.status() != 0:
            raise RuntimeError("tensor-core completion timed out during training")
        if log:
            log(f"epoch {ep + 1}/{epochs}: loss {hist[-1]:.4e} ({time.time() - t0:.1f}s)")
    return hist


def validation_loss(net: WarmStartNet, samples: torch.Tensor) -> dict:
    """Mean loss of the network and of two fixed predictors on held-out samples:
    'zero' (no second difference: the linear extrapolation) and 'previous' (the
    previous second difference: quadratic extrapolation)."""
    out = {"network": 0.0, "zero": 0.0, "previous": 0.0}
    S = samples.shape[0]
    for i in range(S):
        f, t = samples[i, :4], samples[i, 4].float()
        y = net.forward(f)
        out["network"] += 0.5 * float(((y - t) ** 2).mean())
        out["zero"] += 0.5 * float((t**2).mean())
        out["previous"] += 0.5 * float(((f[3].float() - t) ** 2).mean())
    return {k: v / S for k, v in out.items()}


def evaluate(net: WarmStartNet | None, n_particles: int = 10_000_000, steps: int = 30, seed: int = 1234,
             grid: int = GRID, box: float = BOX, dt: float = DT, tol: float = 1e-6, warm_steps: int = 5,
             modes=("plain", "extrapolate", "learned")) -> dict:
    """V-cycles and solve milliseconds per step for each initial guess on one
    held-out collision (same initial conditions for every mode)."""
    icr = random_collision(np.random.default_rng(seed), n_particles, box / grid)
    res = {}
    for mode in modes:
        if mode == "learned" and net is None:
            continue
        eng = _engine(grid, box, tol)
        eng.set_warmstart(mode, net=net if mode == "learned" else None, track=True)
        eng.load(icr.pos, icr.vel, icr.mass, icr.gid)
        eng.prime(dt)
        for _ in range(warm_steps):
            eng.advance(dt)
        eng.ctx.profile_reset()
        eng.ctx.profile(True)
        cycles = []
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        ev0.record()
        for _ in range(steps):
            cycles.append(eng.advance(dt).cycles)
        ev1.record()
        torch.cuda.synchronize()
        stats = eng.ctx.kernel_stats()
        eng.ctx.profile(False)
        solve = sum(v[2] for k, v in stats.items() if k in SOLVE_KERNELS)
        res[mode] = {"mean_vcycles": float(np.mean(cycles)), "vcycles": cycles,
                     "ms_per_solve": solve / steps, "ms_per_step": ev0.elapsed_time(ev1) / steps,
                     "warmstart_ms_per_step": stats.get("warmstart", (0, 0, 0.0))[2] / steps}
        del eng
    res["config"] = {"particles": n_particles, "grid": grid, "steps": steps, "tol": tol, "seed": seed}
    return res


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--runs", type=int, default=200)
    ap.add_argument("--particles", type=int, default=1_000_000)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--every", type=int, default=10)
    ap.add_argument("--epochs", type=int, default=20)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--val-runs", type=int, default=10)
    ap.add_argument("--eval-particles", type=int, default=10_000_000)
    ap.add_argument("--out", default=str(WEIGHTS_PATH))
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args(argv)

    def log(msg):
        print(f"[warmstart] {msg}", flush=True)

    from galaxy_collision_gb300 import _build

    _build.build()
    t0 = time.time()
    train_s = generate_samples(args.runs, args.particles, args.steps, args.every, seed=args.seed, log=log)
    val_s = generate_samples(args.val_runs, args.particles, args.steps, args.every, seed=args.seed + 10_000)
    log(f"{train_s.shape[0]} training / {val_s.shape[0]} validation samples in {time.time() - t0:.0f}s")
    net = WarmStartNet(GRID // 2, seed=args.seed)
    hist = train(net, train_s, args.epochs, args.lr, seed=args.seed, log=log)
    val = validation_loss(net, val_s)
    log(f"validation loss: {val}")
    ev = evaluate(net, args.eval_particles)
    log(f"evaluation: { {k: (v['mean_vcycles'], round(v['ms_per_solve'], 3)) for k, v in ev.items() if k != 'config'} }")
    path = net.save(Path(args.out), train_loss=np.asarray(hist), val_network=val["network"], val_zero=val["zero"],
                    val_previous=val["previous"], runs=args.runs, samples=train_s.shape[0], epochs=args.epochs,
                    lr=args.lr)
    log(f"saved {path}")


if __name__ == "__main__":
    main()

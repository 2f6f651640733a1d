"""Measured engine settings per (device, grid, particle-count bucket), cached in JSON.

Some of the engine's choices change its speed and nothing else (the states are
bit-identical, or every solve still meets the same tolerance): the coarse
multigrid levels by the two persistent cooperative kernels or one launch per
phase (``phase_launches``), and the cell-sort period (``sort_every``, with the
look-ahead at half the period). Which is faster depends on the grid and the
particle count: per-phase launches win at 64^3 and 128^3, the persistent
kernels at 256^3. ``tune`` times every candidate on a short run of a given
state (CUDA events around whole-step graph replays) and caches the fastest
under the key ``<device>/G<grid>/N2^<k>`` (k = floor(log2 particle count)) in
a JSON file: ``$GC_AUTOTUNE_CACHE`` or ``~/.cache/galaxy_collision_gb300/
autotune.json``. ``settings_for`` returns the cached entry or tunes.
"""

from __future__ import annotations

import json
import os
import time
from pathlib import Path

CANDIDATES = (
    {"phase_launches": False, "sort_every": 20},
    {"phase_launches": True, "sort_every": 20},
    {"phase_launches": False, "sort_every": 10},
    {"phase_launches": True, "sort_every": 10},
)


def cache_path() -> Path:
    env = os.environ.get("GC_AUTOTUNE_CACHE")
    return Path(env) if env else Path.home() / ".cache" / "galaxy_collision_gb300" / "autotune.json"


def bucket(n: int) -> int:
    """floor(log2 n): runs within a factor of two share their settings."""
    if n < 1:
        raise ValueError(f"particle count must be positive, got {n}")
    return int(n).bit_length() - 1


def key(device: str, grid: int, n: int) -> str:
    return f"{device}/G{int(grid)}/N2^{bucket(n)}"


def load(path: Path | None = None) -> dict:
    p = path or cache_path()
    try:
        return json.loads(p.read_text())
    except (FileNotFoundError, json.JSONDecodeError):
        return {}


def save(entries: dict, path: Path | None = None) -> None:
    """Write the cache atomically (temporary file, then rename)."""
    p = path or cache_path()
    p.parent.mkdir(parents=True, exist_ok=True)
    tmp = p.with_suffix(p.suffix + f".tmp{os.getpid()}")
    tmp.write_text(json.dumps(entries, indent=1, sort_keys=True))
    tmp.replace(p)


def pick(timings: dict) -> str:
    """The fastest candidate (ties: the first listed)."""
    return min(timings, key=lambda c: (timings[c], list(timings).index(c)))


def _label(c: dict) -> str:
    return ",".join(f"{k}={c[k]}" for k in sorted(c))


def time_candidate(make_engine, state, dt: float, settings: dict, steps: int = 20, warm: int = 3) -> float:
    """ms per step of whole-step graph replays with these settings (the cell
    sorts of the period included), after a prime and `warm` eager steps."""
    import torch

    eng = make_engine(**settings)
    eng.load(*state)
    eng.prime(dt)
    for _ in range(warm):
        eng.advance(dt)
    eng.prepare_graphs(dt)
    eng.advance_graph(dt)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record()
    for _ in range(steps):
        eng.advance_graph(dt)
    ev1.record()
    torch.cuda.synchronize()
    ms = ev0.elapsed_time(ev1) / steps
    del eng
    return ms


def tune(grid: int, n: int, make_engine, state, dt: float, *, device: str, candidates=CANDIDATES, steps: int = 20,
         measure=None, path: Path | None = None) -> dict:
    """Time every candidate and cache the fastest. `measure(settings) -> ms`
    replaces the GPU timing (tests)."""
    measure = measure or (lambda c: time_candidate(make_engine, state, dt, c, steps=steps))
    timings = {}
    by_label = {}
    for c in candidates:
        lab = _label(c)
        by_label[lab] = dict(c)
        timings[lab] = float(measure(dict(c)))
    best = pick(timings)
    entry = {"settings": by_label[best], "ms_per_step": timings, "particles": int(n), "steps": int(steps),
             "tuned_at": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime())}
    entries = load(path)
    entries[key(device, grid, n)] = entry
    save(entries, path)
    return entry


def settings_for(grid: int, n: int, make_engine, state, dt: float, *, device: str, path: Path | None = None,
                 **kw) -> dict:
    """The cached settings for (device, grid, bucket of n), tuned on `state` when absent."""
    entry = load(path).get(key(device, grid, n))
    if entry is None:
        entry = tune(grid, n, make_engine, state, dt, device=device, path=path, **kw)
    return dict(entry["settings"])


__all__ = ["CANDIDATES", "bucket", "key", "load", "save", "pick", "tune", "settings_for", "cache_path",
           "time_candidate"]

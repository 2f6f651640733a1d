"""Shared device contexts for the stateless operators (deposit, grad, gather, kick, drift).

One ``gc_ctx`` per (device, grid size, dx) is cached; the solver and the fused
engine own their own contexts because they keep state between calls.
"""

from __future__ import annotations

import threading

import torch

from galaxy_collision_gb300 import _native

_lock = threading.Lock()
_cache: dict = {}

# Fixed-point resolution of the density deposit: the whole deposited mass is at
# most 2^52 quanta, so a particle's contribution keeps ~1e-8 relative accuracy
# even at 1e8 particles while int64 sums cannot overflow.
DEFAULT_FIXED_POINT_BITS = 52


def op_context(grid_size: int, dx: float) -> _native.Context:
    key = (torch.cuda.current_device(), int(grid_size), float(dx))
    with _lock:
        ctx = _cache.get(key)
        if ctx is None:
            ctx = _native.Context(grid_size, dx, 1.0)
            _cache[key] = ctx
        return ctx


def clear_cache() -> None:
    with _lock:
        for c in _cache.values():
            c.close()
        _cache.clear()

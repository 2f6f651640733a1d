"""Kick-drift-kick leapfrog on the GPU (drop-in for src/galaxy_collision/integrator.py).

:func:`kick` and :func:`drift` are single sm_103a launches with the reference's
f32 arithmetic (``v += a*dt``, ``x += v*dt``, integrator.py:27-59).
:func:`kdk_step` keeps the reference's ordering and cached-acceleration contract
(integrator.py:100-131): ``kick(dt/2) -> drift(dt) -> accel_fn() -> kick(dt/2)``,
one force evaluation per step, ``acc_*`` valid for the current positions on
entry and on exit. The fused engine (:mod:`galaxy_collision_gb300.engine`) runs
the same arithmetic in one particle pass per step.
"""

from __future__ import annotations

from galaxy_collision_gb300._ops import op_context
from galaxy_collision_gb300.data import as_tensor

# Any cached context works for the element-wise kernels; they do not touch the grid.
_ELEMENTWISE_GRID = 2


def _arrays(n, names_and_fields):
    return [as_tensor(f, shape=(n,), name=nm) for nm, f in names_and_fields]


def kick(vel_x, vel_y, vel_z, acc_x, acc_y, acc_z, n: int, dt: float) -> None:
    """Velocity update v += a*dt (call with dt/2 for each leapfrog half-kick)."""
    n = int(n)
    if n <= 0:
        return
    v = _arrays(n, (("vel_x", vel_x), ("vel_y", vel_y), ("vel_z", vel_z)))
    a = _arrays(n, (("acc_x", acc_x), ("acc_y", acc_y), ("acc_z", acc_z)))
    op_context(_ELEMENTWISE_GRID, 1.0).call("gc_kick", *(t.data_ptr() for t in v), *(t.data_ptr() for t in a), n,
                                            float(dt), what="kick")


def drift(pos_x, pos_y, pos_z, vel_x, vel_y, vel_z, n: int, dt: float) -> None:
    """Position update x += v*dt (the full-step drift)."""
    n = int(n)
    if n <= 0:
        return
    p = _arrays(n, (("pos_x", pos_x), ("pos_y", pos_y), ("pos_z", pos_z)))
    v = _arrays(n, (("vel_x", vel_x), ("vel_y", vel_y), ("vel_z", vel_z)))
    op_context(_ELEMENTWISE_GRID, 1.0).call("gc_drift", *(t.data_ptr() for t in p), *(t.data_ptr() for t in v), n,
                                            float(dt), what="drift")


def kdk_step(parts, acc_x, acc_y, acc_z, accel_fn, dt: float) -> None:
    """Advance one KDK leapfrog step with a single acceleration evaluation per step.

    Precondition: ``acc_*`` hold a(x) for the current positions (prime once with
    ``accel_fn()``). Postcondition: ``acc_*`` hold a(x_new). Any out-of-band change
    of positions requires calling ``accel_fn()`` again before the next step.
    """
    n = parts.n
    half = 0.5 * dt
    kick(parts.vel_x, parts.vel_y, parts.vel_z, acc_x, acc_y, acc_z, n, half)
    drift(parts.pos_x, parts.pos_y, parts.pos_z, parts.vel_x, parts.vel_y, parts.vel_z, n, dt)
    accel_fn()
    kick(parts.vel_x, parts.vel_y, parts.vel_z, acc_x, acc_y, acc_z, n, half)


__all__ = ["kick", "drift", "kdk_step"]

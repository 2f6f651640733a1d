"""A bounded device wait that runs out returns a status instead of hanging.

The TMA particle pass and the tensor-core kernels wait on mbarriers with a
clock budget and raise GC_FLAG_TIMEOUT when it is spent. Here the library's own
wait is driven to expiry on an mbarrier that nothing arrives on (a short budget
of 1e6 SM clocks, well under a millisecond), with a positive control where the
arrival happens, and the context is shown to be usable afterwards.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_bounded_wait_expires_and_context_stays_usable(cuda):
    from galaxy_collision_gb300 import _native
    from galaxy_collision_gb300.data import Field, ParticleState
    from galaxy_collision_gb300.deposit import deposit_density

    lib = _native.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    status = torch.zeros(1, dtype=torch.int32, device="cuda")
    # the arrival happens: the wait succeeds and leaves the word alone
    assert lib.gc_selftest_wait_timeout(stream, status.data_ptr(), 1_000_000, 1) == 0
    torch.cuda.synchronize()
    assert int(status.item()) == 0
    # nothing arrives: the wait gives up and reports it
    assert lib.gc_selftest_wait_timeout(stream, status.data_ptr(), 1_000_000, 0) == 0
    torch.cuda.synchronize()
    assert int(status.item()) & _native.GC_FLAG_TIMEOUT
    # out-of-range budgets are refused on the host
    assert lib.gc_selftest_wait_timeout(stream, status.data_ptr(), 0, 0) == _native.GC_ERR_ARG
    assert lib.gc_selftest_wait_timeout(stream, status.data_ptr(), 3_000_000_000, 0) == _native.GC_ERR_ARG
    # the context still works: a deposit gives the oracle's density
    from oracle import pm

    rng = np.random.default_rng(5)
    G, n = 16, 3000
    pos = rng.uniform(0.0, G - 1.0, size=(n, 3)).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)
    p = ParticleState(n)
    for f, a in zip((p.pos_x, p.pos_y, p.pos_z), pos.T):
        f.from_numpy(np.ascontiguousarray(a))
    p.mass.from_numpy(mass)
    rho = Field((G, G, G))
    deposit_density(p, rho, 1.0, fixed_point_bits=52)
    np.testing.assert_array_equal(rho.to_numpy(), pm.deposit_fixed(pos, mass, 1.0, G, 52)[0])

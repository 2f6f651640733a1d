"""The allocation-free deposit entry point (gc_deposit_cic_noalloc).

Some callers cannot allocate device memory where they need a density -- a
memory pool that already owns the whole GPU, a loop that must not take the
device-wide synchronisation of cudaMalloc, or code with no context object to
hold scratch -- so this entry point keeps its scratch in a fixed device array
instead of a gc_ctx. Here it is called through the C ABI, twice in a row on
different inputs and grid sizes (the shared array keeps the previous call's
contents, so the second call checks that it is cleared), and its density must
equal gc_deposit_cic's bit for bit, the tolerance of the other deposit tests.
The file is named to be collected last.
"""

from __future__ import annotations

import ctypes as C

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _arrays(pos, mass):
    cols = [torch.from_numpy(np.ascontiguousarray(pos[:, i])).cuda() for i in range(3)]
    return cols, torch.from_numpy(np.ascontiguousarray(mass)).cuda()


def _reference_density(pos, mass, G, dx, bits):
    from galaxy_collision_gb300.data import Field, ParticleState
    from galaxy_collision_gb300.deposit import deposit_density

    n = pos.shape[0]
    p = ParticleState(n)
    for f, a in zip((p.pos_x, p.pos_y, p.pos_z), pos.T):
        f.from_numpy(np.ascontiguousarray(a))
    p.mass.from_numpy(mass)
    rho = Field((G, G, G))
    deposit_density(p, rho, dx, fixed_point_bits=bits)
    return rho.to_numpy()


def test_noalloc_deposit_matches_context_deposit_twice(cuda):
    from galaxy_collision_gb300 import _native

    lib = _native.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(2024)
    cases = [(64, 0.5, 52, 60000), (24, 1.25, 40, 20000)]
    for G, dx, bits, n in cases:
        pos = rng.uniform(-1.5 * dx, (G + 0.5) * dx, size=(n, 3)).astype(np.float32)
        mass = rng.uniform(0.2, 2.0, size=n).astype(np.float32)
        (x, y, z), m = _arrays(pos, mass)
        rho = torch.full((G, G, G), float("nan"), dtype=torch.float32, device="cuda")
        st = lib.gc_deposit_cic_noalloc(x.data_ptr(), y.data_ptr(), z.data_ptr(), m.data_ptr(), n, G, dx, bits,
                                        rho.data_ptr(), None, stream)
        assert st == 0, lib.gc_last_error(None)
        torch.cuda.synchronize()
        np.testing.assert_array_equal(rho.cpu().numpy(), _reference_density(pos, mass, G, dx, bits))


def test_noalloc_deposit_rejects_grids_beyond_its_scratch(cuda):
    from galaxy_collision_gb300 import _native

    lib = _native.load()
    x = torch.zeros(4, dtype=torch.float32, device="cuda")
    rho = torch.zeros((65, 65, 65), dtype=torch.float32, device="cuda")
    st = lib.gc_deposit_cic_noalloc(x.data_ptr(), x.data_ptr(), x.data_ptr(), x.data_ptr(), 4, 65, 1.0, 52,
                                    rho.data_ptr(), None, None)
    assert st == _native.GC_ERR_ARG
    assert b"grid_size" in lib.gc_last_error(None)


def test_noalloc_deposit_reports_nonfinite_positions(cuda):
    """A NaN position deposits nothing; the caller's device status word gets
    GC_FLAG_NONFINITE_POS (the scratch array's own word is cleared by the next
    call, so the caller passes one of its own), and the rest of the density is
    gc_deposit_cic's."""
    from galaxy_collision_gb300 import _native

    lib = _native.load()
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    rng = np.random.default_rng(7)
    G, dx, bits, n = 16, 1.0, 52, 5000
    pos = rng.uniform(0.0, G - 1.0, size=(n, 3)).astype(np.float32)
    mass = np.full(n, 1.0 / n, np.float32)
    pos[123, 1] = np.nan
    (x, y, z), m = _arrays(pos, mass)
    rho = torch.empty((G, G, G), dtype=torch.float32, device="cuda")
    flags = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = lib.gc_deposit_cic_noalloc(x.data_ptr(), y.data_ptr(), z.data_ptr(), m.data_ptr(), n, G, dx, bits,
                                    rho.data_ptr(), flags.data_ptr(), stream)
    assert st == 0, lib.gc_last_error(None)
    torch.cuda.synchronize()
    assert int(flags.item()) & _native.GC_FLAG_NONFINITE_POS
    # the context deposit skips the same particle (and its mass still sets the quantum)
    np.testing.assert_array_equal(rho.cpu().numpy(), _reference_density(pos, mass, G, dx, bits))
    # finite positions leave the caller's word alone
    flags.zero_()
    pos[123, 1] = 1.0
    (x, y, z), m = _arrays(pos, mass)
    st = lib.gc_deposit_cic_noalloc(x.data_ptr(), y.data_ptr(), z.data_ptr(), m.data_ptr(), n, G, dx, bits,
                                    rho.data_ptr(), flags.data_ptr(), stream)
    assert st == 0, lib.gc_last_error(None)
    torch.cuda.synchronize()
    assert int(flags.item()) == 0

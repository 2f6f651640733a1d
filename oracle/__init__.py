"""CPU oracle of the reference PM hot path -- TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use this package, and only as the checker / the timed CPU
baseline, never as the product path.

* :mod:`oracle.pm` -- ctypes wrapper of ``pm_oracle.c``, the f32 restatement of
  the reference's Taichi kernels (deposit, grad, gather, kick, drift, the
  reference multigrid) plus the FP64 and fixed-point deposit variants.
* :mod:`oracle.fft` -- NumPy restatement of the reference's zero-padded FFT
  oracle (src/galaxy_collision/solver/fft_oracle.py:54-109).
* :mod:`oracle.dst` -- exact FP64 solve of the same discrete Dirichlet problem
  (7-point Laplacian, given faces) by the type-I sine transform.
* :mod:`oracle.diagnostics` -- host FP64 diagnostics (src/galaxy_collision/diagnostics.py).
* :mod:`oracle.samplers` -- none; the initial conditions are product code.

Parity pinning: the restatement is checked against the reference's own
known-answer tests (tests/test_deposit.py, test_integrator.py,
test_solver_multigrid.py, test_solver_fft.py, test_diagnostics.py) and against
fixtures generated by importing the reference's pure-NumPy modules
(``tests/golden/make_golden.py``). The Taichi kernels themselves cannot run here
(Taichi is not installed), so bitwise parity with the Taichi backend is not
pinned; the tolerances of the reference's own tests are.
"""

"""GB300-native particle-mesh force chain with the Python surface of the
reference package ``galaxy_collision`` (pouyalj/Galaxy-Collision-with-CUDA-FFT).

The hot path (CIC deposit, open-boundary multigrid Poisson solve, -grad(phi),
CIC gather, KDK kick/drift) runs in hand-written sm_103a CUDA kernels behind the
C ABI of ``include/gcpm.h``; this package holds the host-side mirror of the
reference interface (``deposit``, ``integrator``, ``solver``,
``diagnostics_device``, ``data``, ``config``, ``io``, ``bench``) and the fused
engine (``engine``). There is no CPU fallback.
"""

__version__ = "0.1.0"

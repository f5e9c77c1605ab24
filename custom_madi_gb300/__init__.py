"""GB300-native MADI Monte Carlo diffusion hot path (drop-in for the reference's madi package).

Submodules mirror the reference package: config, ensemble, walker_gpu, signal,
library, fitters_gpu.  Compute runs in hand-written sm_103a CUDA kernels behind
the C ABI of include/madi_gb300.h (loaded by _native.py).
"""

from . import config  # noqa: F401

__all__ = ["config", "ensemble", "walker_gpu", "signal", "library", "fitters_gpu"]
__version__ = "0.1.0"

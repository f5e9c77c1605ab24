"""GB300-native MADI Monte Carlo diffusion hot path (drop-in for the reference's madi package).

Submodules mirror the reference package: config, ensemble, walker_gpu, signal,
library, fitters_gpu, fitters.  Compute runs in hand-written sm_103a CUDA
kernels behind the C ABI of include/madi_gb300.h (loaded by _native.py on first
use; importing the package loads no native code).

``install_madi_alias()`` registers this package under the reference's name, so
``import madi`` and ``from madi.walker_gpu import run_walk_Y`` resolve here.
"""

import sys

from . import config  # noqa: F401
from . import ensemble  # noqa: F401
from . import walker_gpu  # noqa: F401
from . import signal  # noqa: F401
from . import library  # noqa: F401
from . import fitters_gpu  # noqa: F401
from . import fitters  # noqa: F401

__all__ = ["config", "ensemble", "walker_gpu", "signal", "library", "fitters_gpu", "fitters", "install_madi_alias"]
__version__ = "0.2.0"

_ALIASED = ("config", "ensemble", "walker_gpu", "signal", "library", "fitters_gpu", "fitters")


def install_madi_alias(name: str = "madi") -> None:
    """Make ``import madi`` (and ``madi.<submodule>``) resolve to this package.

    Raises if another package of that name is already imported: mixing the
    reference and this package in one process would silently pick one of them.
    """
    this = sys.modules[__name__]
    have = sys.modules.get(name)
    if have is not None and have is not this:
        raise RuntimeError(f"a different module is already imported as {name!r}: {getattr(have, '__file__', have)}")
    sys.modules[name] = this
    for sub in _ALIASED:
        sys.modules[f"{name}.{sub}"] = sys.modules[f"{__name__}.{sub}"]

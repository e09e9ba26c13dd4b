"""GB300-native (sm_103a) implementation of QuTiP's time-evolution hot path.

The compute path is hand-written CUDA in ``csrc/`` behind the C ABI declared in
``include/qutip_gb300.h`` and loaded with ctypes; there is no CPU fallback.
"""
__version__ = "0.1.0"

from . import coefficients, systems, vern7_tableau  # noqa: F401  (no GPU needed)
from .coefficients import Coefficient, coefficient  # noqa: F401


def __getattr__(name):
    # Device-side modules import torch and load the CUDA library lazily.
    import importlib
    if name in ("operator", "vern7", "solver", "batched", "serving", "superop", "qutip_plugin",
                "_lib"):
        return importlib.import_module(f"{__name__}.{name}")
    if name in ("mesolve", "solve_system"):
        return getattr(importlib.import_module(f"{__name__}.solver"), name)
    raise AttributeError(name)

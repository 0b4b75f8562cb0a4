"""GB300 particle-mesh engine: Python host layer over libpm_gb300.so.

``PMContext`` exposes the reference's per-step functions (density, fourier_grid,
potential, integrate, advance_time) on device tensors; ``Batch`` advances many resident
simulations together; ``build()`` compiles the CUDA library in-tree.
"""
from .build import LIB, build  # noqa: F401
from .config import Config, step_count  # noqa: F401
from ._lib import PMError  # noqa: F401


def __getattr__(name):
    # torch-dependent pieces are imported lazily so that build() works without a GPU
    if name == "PMContext":
        from .context import PMContext
        return PMContext
    if name == "Batch":
        from .batch import Batch
        return Batch
    raise AttributeError(name)

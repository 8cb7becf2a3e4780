"""tmv_gb300: TMV's dense hot path (blocked product, partial-pivoting LU
factor and solve) as hand-written sm_103a CUDA behind a C ABI (include/tmvg.h).

Importing the package does not touch the GPU.  The compiled library
tmv_gb300/_build/libtmvg.so is loaded on first use; when it is missing the
first call raises ImportError (there is no CPU fallback).
"""
from ._lib import LIB_PATH, SingularError, TmvgError  # noqa: F401

__version__ = "0.1.0"


def __getattr__(name):
    # Lazy submodules so that `import tmv_gb300` works without torch/CUDA.
    if name in ("linalg", "matrix", "mixed", "batched", "adjoint"):
        import importlib

        return importlib.import_module(f".{name}", __name__)
    raise AttributeError(name)

"""Loader of the native engine.

The product path has no fallback: if the CUDA extension is missing, importing
it raises ImportError with the build command, and every operation that
reaches a GPU without one raises the engine's PLException.
"""
import importlib
import os
import sys

_PKG = os.path.dirname(os.path.abspath(__file__))
_mod = None


def native():
    """Return the ``lightning_gpu_qubit_ops`` extension module (built in-tree)."""
    global _mod
    if _mod is None:
        try:
            _mod = importlib.import_module("pennylane_lightning_gpu_gb300.lightning_gpu_qubit_ops")
        except ImportError as e:  # pragma: no cover - exercised when the build is missing
            raise ImportError(
                "The GB300 engine extension is not built. Run "
                "`python -c 'import __graft_entry__ as g; g.build()'` from the repository root "
                "(it compiles the sm_103a kernels and the pybind11 module in-tree)."
            ) from e
    return _mod


def library_path():
    return os.path.join(_PKG, "_lib", "liblgpu_gb300.so")


def build(verbose=False):
    from . import _build

    return _build.build(verbose=verbose)

"""GB300-native statevector engine with the LightningGPU hot-path interface.

* ``lightning_gpu_qubit_ops`` — pybind11 module with the drop-in classes
  ``LightningGPU_C64/C128``, the observable family, ``OpsStructGPU_*`` and
  ``AdjointJacobianGPU_*`` (same names as the reference module).
* ``LightningGPU`` — the Python device with ``apply``, ``expval``, ``var``,
  ``probability``, ``generate_samples``, ``adjoint_jacobian`` and ``vjp``.
* ``batched`` / ``serving`` / ``torch_adjoint`` — batched persistent
  execution, the continuous-batching server and the autograd adjoint.
"""
from ._native import build, library_path, native  # noqa: F401
from ._version import __version__  # noqa: F401


def __getattr__(name):
    # Lazy access so that ``import pennylane_lightning_gpu_gb300`` works for
    # build-only uses without loading the extension.
    if name == "lightning_gpu_qubit_ops":
        return native()
    if name in ("LightningGPU",):
        from .lightning_gpu import LightningGPU

        return LightningGPU
    raise AttributeError(name)

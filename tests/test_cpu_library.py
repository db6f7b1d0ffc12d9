"""CPU-side checks of the native library: it builds, loads, exports every
entry point that include/lgpu.h declares, and fails loudly without a GPU."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    with open(os.path.join(ROOT, "include", "lgpu.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"\b(lgpu_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_entry_points():
    syms = _declared_symbols()
    for s in ["lgpu_apply_matrix", "lgpu_apply_pauli_rotation", "lgpu_expval_matrix", "lgpu_expval_pauli_words",
              "lgpu_probs", "lgpu_sample", "lgpu_dot", "lgpu_axpy", "lgpu_adjoint_step", "lgpu_apply_fused_block"]:
        assert s in syms


def test_library_exports_every_declared_symbol(native):
    import pennylane_lightning_gpu_gb300 as pkg

    lib = ctypes.CDLL(pkg.library_path())
    missing = [s for s in _declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_library_reports_errors_without_device(native):
    import pennylane_lightning_gpu_gb300 as pkg

    lib = ctypes.CDLL(pkg.library_path())
    lib.lgpu_last_error_string.restype = ctypes.c_char_p
    # invalid arguments are rejected before any CUDA call
    rc = lib.lgpu_set_basis(None, 3, 1, 0, ctypes.c_double(1.0), ctypes.c_double(0.0), None)
    assert rc == 1
    assert b"null" in lib.lgpu_last_error_string()
    assert lib.lgpu_abi_version() == 1


def test_module_classes(native):
    for name in ["LightningGPU_C64", "LightningGPU_C128", "NamedObsGPU_C128", "HermitianObsGPU_C128",
                 "TensorProdObsGPU_C128", "HamiltonianGPU_C128", "SparseHamiltonianGPU_C128", "OpsStructGPU_C128",
                 "AdjointJacobianGPU_C128", "DevPool", "DevTag", "PLException", "device_reset", "allToAllAccess",
                 "is_gpu_supported", "get_gpu_arch"]:
        assert hasattr(native, name), name


def test_gpu_use_fails_loudly_without_gpu(native):
    try:
        import torch

        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(native.PLException):
        native.LightningGPU_C128(3)

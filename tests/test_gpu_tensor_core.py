"""Dense 6-target complex64 gates on the tensor cores (tcgen05) against the
oracle and against the FP32 shared-memory kernel.

Tolerance: complex64 1e-5 absolute per amplitude against the FP64 oracle (the
three-TF32-product scheme carries about 2^-22 of each column's size).
"""
import numpy as np
import pytest

from helpers import make_sv, random_state, random_unitary

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [12, 13, 17, 21])
@pytest.mark.parametrize("adjoint", [False, True])
def test_dense6_low_bits_on_tensor_cores(native, oracle, n, adjoint):
    rng = np.random.default_rng(600 + n + 7 * adjoint)
    psi = random_state(n, rng)
    u = random_unitary(64, rng)
    wires = [int(w) for w in rng.permutation(np.arange(n - 6, n))]  # the six lowest state bits, any order
    assert native.get_tensor_mode() == 1
    sv = make_sv(native, "c64", psi)
    sv.apply("QubitUnitary", wires, adjoint, [], u.ravel())
    got = sv.GetState().astype(np.complex128)
    ref = oracle.apply_ops(psi, [("QubitUnitary", wires, [], adjoint, u)])
    assert np.max(np.abs(got - ref)) < 1e-5
    native.set_tensor_mode(0)
    try:
        sv2 = make_sv(native, "c64", psi)
        sv2.apply("QubitUnitary", wires, adjoint, [], u.ravel())
        simt = sv2.GetState().astype(np.complex128)
    finally:
        native.set_tensor_mode(1)
    assert np.max(np.abs(simt - ref)) < 1e-5
    assert np.max(np.abs(got - simt)) < 1e-5


def test_dense6_general_matrix_and_repeated_calls(native, oracle):
    """A non-unitary matrix with entries of very different sizes, applied
    twice in a row (the kernel keeps no state between launches)."""
    rng = np.random.default_rng(5)
    n = 14
    psi = random_state(n, rng)
    m = (rng.normal(size=(64, 64)) + 1j * rng.normal(size=(64, 64))) / 8.0
    m[:, 3] *= 1e-3
    wires = list(range(n - 6, n))
    sv = make_sv(native, "c64", psi)
    for _ in range(2):
        sv.apply("QubitUnitary", wires, False, [], m.ravel())
    ref = oracle.apply_ops(psi, [("QubitUnitary", wires, [], False, m)] * 2)
    scale = max(1.0, float(np.max(np.abs(ref))))
    assert np.max(np.abs(sv.GetState() - ref)) < 1e-5 * scale


def test_tensor_mode_rejects_bad_values(native):
    with pytest.raises(native.PLException):
        native.set_tensor_mode(2)
    assert native.get_tensor_mode() == 1


def test_dense6_long_pipeline_matches_fp32_kernel(native):
    """24 qubits: each CTA runs dozens of units through the two-slot pipeline;
    the result equals the FP32 shared-memory kernel's (itself checked against
    the oracle by test_dense_matrix) within the complex64 tolerance."""
    rng = np.random.default_rng(24)
    n = 24
    psi = random_state(n, rng).astype(np.complex64)
    u = random_unitary(64, rng)
    wires = list(range(n - 1, n - 7, -1))
    sv = make_sv(native, "c64", psi)
    sv.apply("QubitUnitary", wires, False, [], u.ravel())
    got = sv.GetState()
    native.set_tensor_mode(0)
    try:
        sv2 = make_sv(native, "c64", psi)
        sv2.apply("QubitUnitary", wires, False, [], u.ravel())
        ref = sv2.GetState()
    finally:
        native.set_tensor_mode(1)
    assert np.max(np.abs(got - ref)) < 1e-5
    assert abs(np.linalg.norm(got.astype(np.complex128)) - np.linalg.norm(psi.astype(np.complex128))) < 1e-5

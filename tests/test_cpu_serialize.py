"""Serialisation of tapes for the adjoint method (the reference's
_serialize.py:158-336 behaviour), on the host: observable classes per dtype,
wire mapping, Hamiltonians split into one observable per term with the
offsets that fold the Jacobian rows back, refusals, and the operation lists
(bound gates by name, others by matrix, Rot/CRot expanded)."""
import numpy as np
import pytest

from pennylane_lightning_gpu_gb300 import _serialize as S
from pennylane_lightning_gpu_gb300 import ops as Q


def _tape(ops, obs):
    return Q.QuantumTape(ops, [Q.expval(o) for o in obs])


@pytest.mark.parametrize("single", [False, True])
def test_observables_and_offsets(native, single):
    suf = "C64" if single else "C128"
    wm = {"a": 0, "b": 1, "c": 2, "d": 3}
    H = Q.Hamiltonian([0.5, -1.5, 2.0], [Q.PauliZ("a") @ Q.PauliX("d"), Q.PauliY("b"), Q.Identity("c")])
    tape = _tape([], [Q.PauliX("b"), H, Q.PauliZ("c") @ Q.Hadamard("d")])
    out, offsets = S._serialize_observables(tape, wm, use_csingle=single)
    assert offsets == [0, 1, 4, 5]
    assert [type(o).__name__ for o in out] == ["NamedObsGPU_" + suf] + ["HamiltonianGPU_" + suf] * 3 + [
        "TensorProdObsGPU_" + suf]
    assert repr(out[0]) == "PauliX[1]"
    assert out[0].get_wires() == [1]
    assert "0.5" in repr(out[1]) and "PauliZ[0] @ PauliX[3]" in repr(out[1])
    assert "-1.5" in repr(out[2]) and "PauliY[1]" in repr(out[2])
    assert "Identity[2]" in repr(out[3])
    # unsplit: one Hamiltonian
    out2, offsets2 = S._serialize_observables(tape, wm, use_csingle=single, split_terms=False)
    assert offsets2 == [0, 1, 2, 3] and type(out2[1]).__name__ == "HamiltonianGPU_" + suf


def test_hermitian_refused_unless_allowed(native):
    herm = Q.Hermitian(np.array([[1.0, 2j], [-2j, 0.5]]), [1])
    tape = _tape([], [herm])
    with pytest.raises(TypeError, match="Hermitian observables are not currently supported"):
        S._serialize_observables(tape, {0: 0, 1: 1})
    out, _ = S._serialize_observables(tape, {0: 0, 1: 1}, allow_hermitian=True)
    assert type(out[0]).__name__ == "HermitianObsGPU_C128" and out[0].get_wires() == [1]
    with pytest.raises(TypeError, match="Hermitian"):
        S._serialize_observables(_tape([], [Q.PauliX(0) @ herm]), {0: 0, 1: 1})


def test_operations_bound_by_name_or_matrix(native):
    u = np.linalg.qr(np.arange(16).reshape(4, 4) + 1j * np.eye(4))[0]
    ops = [Q.BasisState([1], [0]), Q.op("RX", 1, 0.3), Q.op("CNOT", [0, 1]), Q.QubitUnitary(u, [1, 0]),
           Q.op("Rot", 0, 0.1, 0.2, 0.3), Q.op("CRot", [1, 0], 0.4, 0.5, 0.6).adjoint(),
           Q.op("IsingZZ", [0, 1], 0.7).adjoint()]
    tape = _tape(ops, [Q.PauliZ(0)])
    (names, params, wires, inverses, mats), uses_prep = S._serialize_ops(tape, {0: 0, 1: 1})
    assert uses_prep
    assert names == ["RX", "CNOT", "QubitUnitary", "RZ", "RY", "RZ", "CRZ", "CRY", "CRZ", "IsingZZ"]
    assert [list(p) for p in params][:1] == [[0.3]] and len(params[2]) == 0
    assert np.allclose(mats[2].reshape(4, 4), u) and all(len(m) == 0 for i, m in enumerate(mats) if i != 2)
    # Rot = RZ(phi) RY(theta) RZ(omega); an inverted CRot = inverted factors in reverse order
    assert [float(p[0]) for p in params[3:6]] == pytest.approx([0.1, 0.2, 0.3])
    assert [float(p[0]) for p in params[6:9]] == pytest.approx([0.6, 0.5, 0.4])
    assert inverses == [False, False, False, False, False, False, True, True, True, True]
    assert wires[6] == [1, 0] and wires[2] == [1, 0]
    # parameter positions: the inverted CRot block comes out reversed
    assert S._expanded_param_positions(tape) == [0, 1, 2, 3, 6, 5, 4, 7]


def test_hamiltonian_wires_in_order_of_appearance():
    H = Q.Hamiltonian([1.0, 2.0], [Q.PauliZ("b") @ Q.PauliX(3), Q.PauliY(0)])
    assert H.wires == ["b", 3, 0]
    m = H.matrix(["b", 3, 0])
    z, x, y = np.diag([1.0, -1.0]), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]])
    assert np.allclose(m, np.kron(np.kron(z, x), np.eye(2)) + 2 * np.kron(np.eye(4), y))

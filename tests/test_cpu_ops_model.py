"""The Python op model's matrices agree with the oracle's named gates."""
import numpy as np
import pytest

from pennylane_lightning_gpu_gb300 import ops as Q

GATES = [("PauliX", 1, 0), ("PauliY", 1, 0), ("PauliZ", 1, 0), ("Hadamard", 1, 0), ("S", 1, 0), ("T", 1, 0),
         ("RX", 1, 1), ("RY", 1, 1), ("RZ", 1, 1), ("PhaseShift", 1, 1), ("Rot", 1, 3), ("CNOT", 2, 0), ("CY", 2, 0),
         ("CZ", 2, 0), ("SWAP", 2, 0), ("CRX", 2, 1), ("CRY", 2, 1), ("CRZ", 2, 1), ("CRot", 2, 3),
         ("ControlledPhaseShift", 2, 1), ("IsingXX", 2, 1), ("IsingYY", 2, 1), ("IsingZZ", 2, 1),
         ("SingleExcitation", 2, 1), ("SingleExcitationMinus", 2, 1), ("SingleExcitationPlus", 2, 1),
         ("CSWAP", 3, 0), ("Toffoli", 3, 0), ("DoubleExcitation", 4, 1), ("DoubleExcitationMinus", 4, 1),
         ("DoubleExcitationPlus", 4, 1), ("MultiRZ", 3, 1)]


@pytest.mark.parametrize("name,nw,npar", GATES)
def test_matrix_matches_oracle(oracle, name, nw, npar):
    rng = np.random.default_rng(1)
    n = 5
    wires = [int(x) for x in rng.choice(n, size=nw, replace=False)]
    params = list(rng.uniform(0, 2 * np.pi, npar))
    psi = rng.normal(size=32) + 1j * rng.normal(size=32)
    psi /= np.linalg.norm(psi)
    o = Q.op(name, wires, *params)
    a = oracle.apply_ops(psi, [(name, wires, params, False, None)])
    b = oracle.apply_ops(psi, [("QubitUnitary", wires, [], False, o.matrix())])
    assert np.allclose(a, b, atol=1e-13)
    c = oracle.apply_ops(psi, [(name, wires, params, True, None)])
    d = oracle.apply_ops(psi, [("QubitUnitary", wires, [], False, o.adjoint().matrix())])
    assert np.allclose(c, d, atol=1e-13)


def test_tensor_and_hamiltonian_matrices():
    h = Q.Hamiltonian([0.5, -1.0], [Q.PauliZ(0) @ Q.PauliX(2), Q.PauliY(1)])
    m = h.matrix(wire_order=[0, 1, 2])
    z, x, y, i2 = np.diag([1, -1]), np.array([[0, 1], [1, 0]]), np.array([[0, -1j], [1j, 0]]), np.eye(2)
    ref = 0.5 * np.kron(np.kron(z, i2), x) - np.kron(np.kron(i2, y), i2)
    assert np.allclose(m, ref)


def test_tape_parameter_bookkeeping():
    tape = Q.QuantumTape([Q.StatePrep([1, 0], [0]), Q.op("RX", 0, 0.1), Q.op("Rot", 0, 0.2, 0.3, 0.4)],
                         [Q.expval(Q.PauliZ(0))])
    assert tape.trainable_params == [0, 1, 2, 3]
    o, k, j = tape.get_operation(2)
    assert o.name == "Rot" and j == 1


@pytest.mark.parametrize("name,wires", [("Rot", [1]), ("CRot", [2, 0])])
@pytest.mark.parametrize("inverse", [False, True])
def test_rot_expansion_is_exact(name, wires, inverse):
    """The adjoint method's one-parameter expansion of Rot/CRot (and their
    inverses) multiplies back to the gate, and the parameter positions it
    reports follow the expanded order."""
    from pennylane_lightning_gpu_gb300._serialize import _expand_rot, _expanded_param_positions

    o = Q.op(name, wires, 0.3, -1.1, 2.4)
    if inverse:
        o = o.adjoint()
    parts = _expand_rot(o)
    u = np.eye(1 << len(wires), dtype=complex)
    for p in parts:
        u = p.matrix() @ u
    assert np.allclose(u, o.matrix(), atol=1e-14)
    tape = Q.QuantumTape([Q.op("RX", 0, 0.1), o, Q.op("RY", 1, 0.2)], [Q.expval(Q.PauliZ(0))])
    pos = _expanded_param_positions(tape)
    assert pos == ([0, 3, 2, 1, 4] if inverse else [0, 1, 2, 3, 4])
    expanded = [pp for p in parts for pp in p.parameters]
    assert [expanded[pos[q] - 1] for q in (1, 2, 3)] == o.parameters

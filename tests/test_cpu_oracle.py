"""The oracle against closed forms (the reference's own known answers are in
test_cpu_golden.py)."""
import numpy as np
import pytest


def test_rx_closed_form(oracle):
    t = 0.37
    s = oracle.run(1, [("RX", [0], [t], False, None)])
    assert np.allclose(s, [np.cos(t / 2), -1j * np.sin(t / 2)], atol=1e-15)


def test_bell_and_wire_order(oracle):
    s = oracle.run(2, [("Hadamard", [0], [], False, None), ("CNOT", [0, 1], [], False, None)])
    assert np.allclose(s, [1 / np.sqrt(2), 0, 0, 1 / np.sqrt(2)])
    # wire 0 is the most significant bit: X on wire 0 of |00> gives index 2
    s = oracle.run(2, [("PauliX", [0], [], False, None)])
    assert s[2] == 1


def test_probability_lsb_first(oracle):
    s = oracle.run(3, [("PauliX", [0], [], False, None)])  # |100>
    # output bit k <-> wires[k]: wires [0, 2] -> index 1 (bit 0 from wire 0)
    p = oracle.probs(s, [0, 2])
    assert p[1] == 1.0


def test_sample_decode(oracle):
    idx = np.array([0, 5, 6], np.uint64)
    bits = oracle.decode_samples(idx, 3)
    assert bits.tolist() == [[0, 0, 0], [1, 0, 1], [1, 1, 0]]


def test_adjoint_closed_forms(oracle):
    p = 0.4
    s = oracle.run(1, [("RX", [0], [p], False, None)])
    jac = oracle.adjoint_jacobian(s, [("RX", [0], [p], False, None)], [(False, [(1.0, [("PauliZ", [0], None)])])], [0])
    assert abs(jac[0, 0] + np.sin(p)) < 1e-14
    s = oracle.run(1, [("RY", [0], [p], False, None)])
    jac = oracle.adjoint_jacobian(s, [("RY", [0], [p], False, None)], [(False, [(1.0, [("PauliX", [0], None)])])], [0])
    assert abs(jac[0, 0] - np.cos(p)) < 1e-14


def test_unsupported_gate(oracle):
    with pytest.raises(oracle.OracleError, match="Currently unsupported gate: Foo"):
        oracle.run(1, [("Foo", [0], [], False, None)])


def test_rot_adjoint_quirk_differs(oracle):
    """Adjoint(Rot) of the reference equals Rot(omega,theta,phi)^dag, not the inverse."""
    ops = [("Rot", [0], [0.3, 0.7, 1.9], False, None), ("Rot", [0], [0.3, 0.7, 1.9], True, None)]
    s = oracle.run(1, ops)
    assert np.allclose(s, [1, 0])  # mathematical inverse (default)
    oracle.set_rot_quirk(True)
    try:
        q = oracle.run(1, ops)
    finally:
        oracle.set_rot_quirk(False)
    assert np.max(np.abs(q - s)) > 0.1

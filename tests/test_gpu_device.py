"""The Python LightningGPU device end to end against the oracle.

Tolerances: complex128 1e-10 (expvals, states, Jacobians), complex64 1e-5;
central differences (h = 1e-4, complex128) agree with the adjoint to 1e-7.
"""
import numpy as np
import pytest

from pennylane_lightning_gpu_gb300 import ops as Q
from pennylane_lightning_gpu_gb300 import workloads

pytestmark = pytest.mark.gpu


def _dev(n, dtype=np.complex128, **kw):
    from pennylane_lightning_gpu_gb300.lightning_gpu import LightningGPU

    return LightningGPU(n, c_dtype=dtype, **kw)


def _oracle_ops(tape_ops):
    out = []
    for o in tape_ops:
        if isinstance(o, Q.Adjoint):
            out.append((o.name, o.wires, o.parameters, True, o.base._matrix))
        else:
            out.append((o.name, o.wires, o.parameters, False, o._matrix))
    return out


def _ops(n, rng, layers=2):
    ops = [Q.op(*o[:2], *o[2]) for o in workloads.random_circuit(n, layers, rng)]
    ops.append(Q.op("IsingYY", [0, 1], 0.37).adjoint())
    ops.append(Q.QubitUnitary(np.linalg.qr(rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4)))[0], [2, 0]))
    return ops


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-10), (np.complex64, 1e-5)])
def test_execute_measurements(oracle, dtype, tol):
    rng = np.random.default_rng(0)
    n = 6
    ops = _ops(n, rng)
    H = Q.Hamiltonian([0.3, -0.8, 0.25], [Q.PauliZ(0) @ Q.PauliX(3), Q.PauliY(1), Q.PauliZ(5)])
    herm = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    herm = herm + herm.conj().T
    tape = Q.QuantumTape(ops, [Q.expval(Q.PauliX(2)), Q.expval(H), Q.var(Q.PauliY(4)),
                               Q.expval(Q.Hermitian(herm, [1, 4])), Q.probs([0, 2, 3]),
                               Q.expval(Q.Projector([1, 0], [2, 3]))])
    dev = _dev(n, dtype)
    res = dev.execute(tape)
    psi = oracle.run(n, _oracle_ops(ops))
    assert abs(res[0] - oracle.expval_matrix(psi, np.array([[0, 1], [1, 0]]), [2]).real) < tol
    assert abs(res[1] - oracle.expval_matrix(psi, H.matrix(list(range(n))), list(range(n))).real) < tol * 10
    y = np.array([[0, -1j], [1j, 0]])
    v = 1 - oracle.expval_matrix(psi, y, [4]).real ** 2
    assert abs(res[2] - v) < tol * 10
    assert abs(res[3] - oracle.expval_matrix(psi, herm, [1, 4]).real) < tol * 10
    # probabilities in PennyLane order (first wire most significant)
    p = oracle.probs(psi, [0, 2, 3]).reshape(2, 2, 2).transpose().reshape(-1)
    assert np.max(np.abs(res[4] - p)) < tol
    p23 = oracle.probs(psi, [2, 3]).reshape(2, 2).T.reshape(-1)  # PennyLane order over wires [2, 3]
    assert abs(res[5] - p23[0b10]) < tol


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-10), (np.complex64, 1e-5)])
def test_var_observables(oracle, dtype, tol):
    """var = <O^2> - <O>^2 for one-wire Paulis, tensor products (X (x) Y and
    Z (x) H (x) Y) and a 2-wire Hermitian after rotations, against the oracle
    (lightning_gpu.py:936-960)."""
    rng = np.random.default_rng(41)
    n = 4
    ops = [Q.op("RX", 0, 0.43), Q.op("RY", 1, -1.2), Q.op("RX", 2, 2.1), Q.op("CNOT", [0, 1]),
           Q.op("RZ", 2, 0.77), Q.op("RY", 3, 0.35), Q.op("CNOT", [2, 3])]
    herm = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    herm = herm + herm.conj().T
    observables = [Q.PauliZ(0), Q.PauliX(1) @ Q.PauliY(2), Q.PauliZ(0) @ Q.Hadamard(1) @ Q.PauliY(3),
                   Q.Hermitian(herm, [3, 1])]
    dev = _dev(n, dtype)
    res = dev.execute(Q.QuantumTape(ops, [Q.var(o) for o in observables]))
    psi = oracle.run(n, _oracle_ops(ops))
    for got, o in zip(res, observables):
        m = o.matrix()
        w = list(o.wires)
        mean = oracle.expval_matrix(psi, m, w).real
        sq = oracle.expval_matrix(psi, m.conj().T @ m, w).real
        scale = max(1.0, float(np.abs(m).max()) ** 2)
        assert abs(got - (sq - mean ** 2)) < tol * 10 * scale, (o, got, sq - mean ** 2)


def test_state_prep_and_basis_state(oracle):
    rng = np.random.default_rng(1)
    n = 5
    dev = _dev(n)
    sub = rng.normal(size=4) + 1j * rng.normal(size=4)
    sub /= np.linalg.norm(sub)
    dev.apply([Q.StatePrep(sub, [3, 1]), Q.op("RX", 2, 0.4)])
    full = np.zeros(32, complex)
    for k in range(4):
        idx = ((k >> 1) & 1) << (n - 1 - 3) | (k & 1) << (n - 1 - 1)
        full[idx] = sub[k]
    ref = oracle.apply_ops(full, [("RX", [2], [0.4], False, None)])
    assert np.allclose(dev.state, ref, atol=1e-12)
    dev.reset()
    dev.apply([Q.BasisState([1, 0, 1], [0, 2, 4])])
    st = dev.state
    assert st[0b10001] == 1  # wires 0 and 4 set: bits 4 and 0
    with pytest.raises(Exception):
        dev.apply([Q.op("RX", 0, 0.1), Q.BasisState([1], [0])])


def test_samples_and_shot_expval():
    n = 3
    dev = _dev(n, shots=20000, seed=11)
    ops = [Q.op("RY", 0, 1.1), Q.op("CNOT", [0, 1]), Q.op("RX", 2, 0.6)]
    dev.reset()
    dev.apply(ops)
    s = dev.generate_samples()
    assert s.shape == (20000, n) and set(np.unique(s)) <= {0, 1}
    assert np.all(s[:, 0] == s[:, 1])
    tape = Q.QuantumTape(ops, [Q.expval(Q.PauliZ(0)), Q.expval(Q.PauliX(2))])
    r = dev.execute(tape)
    assert abs(r[0] - np.cos(1.1)) < 0.03
    assert abs(r[1]) < 0.03


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
def test_sample_dimensions_and_values(dtype):
    """The scenarios of the reference's tests/test_sample.py:43-100: the
    shot count may change between draws, samples of PauliZ and of a tensor
    product have one entry per shot, and every sample is +1 or -1."""
    dev = _dev(2, dtype, shots=1000, seed=5)
    dev.apply([Q.op("RX", 0, 1.5708), Q.op("RX", 1, 1.5708)])
    for shots, obs in ((10, Q.PauliZ(0)), (12, Q.PauliZ(1)), (17, Q.PauliX(0) @ Q.PauliZ(1))):
        dev.reset()
        dev.apply([Q.op("RX", 0, 1.5708), Q.op("RX", 1, 1.5708)])
        dev.shots = shots
        dev._samples = dev.generate_samples()
        s = dev.sample(obs)
        assert s.shape == (shots,)
        assert np.allclose(s ** 2, 1)
    dev.reset()
    dev.shots = 1000
    dev.apply([Q.op("RX", 0, 1.5708)])
    dev._samples = dev.generate_samples()
    s = dev.sample(Q.PauliZ(0))
    assert np.allclose(s ** 2, 1) and abs(np.mean(s)) < 0.15


@pytest.mark.parametrize("split", [False, True])
def test_adjoint_jacobian_vs_oracle_and_fd(oracle, split):
    rng = np.random.default_rng(2)
    n = 5
    ops = [Q.op("RX", w, rng.uniform(0, 6)) for w in range(n)]
    ops += [Q.op("CNOT", [0, 1]), Q.op("CRY", [1, 3], 0.7), Q.op("Rot", 2, 0.1, 0.8, -0.4),
            Q.op("IsingZZ", [2, 4], 1.3), Q.op("PhaseShift", 0, 0.5).adjoint(), Q.op("SingleExcitation", [3, 4], 0.9)]
    H = Q.Hamiltonian([0.4, -1.2, 0.7], [Q.PauliZ(0) @ Q.PauliZ(1), Q.PauliX(3), Q.PauliY(2) @ Q.PauliZ(4)])
    tape = Q.QuantumTape(ops, [Q.expval(Q.PauliZ(2)), Q.expval(H)])
    dev = _dev(n)
    jac = dev.adjoint_jacobian(tape, split_terms=split)
    # central differences on the device
    params = [p for o in ops for p in o.parameters]

    def f(ps):
        k = 0
        new = []
        for o in ops:
            m = len(o.parameters)
            base = Q.Operation(o.name, o.wires, ps[k:k + m], o._matrix)
            new.append(base.adjoint() if isinstance(o, Q.Adjoint) else base)
            k += m
        return np.array(dev.execute(Q.QuantumTape(new, tape.measurements)))

    h = 1e-4
    fd = np.zeros_like(jac)
    for i in range(len(params)):
        e = np.zeros(len(params))
        e[i] = h
        fd[:, i] = (f(np.array(params) + e) - f(np.array(params) - e)) / (2 * h)
    assert np.max(np.abs(jac - fd)) < 1e-7
    # oracle adjoint on the serialised (Rot-expanded) ops
    from pennylane_lightning_gpu_gb300._serialize import _expand_rot

    flat = []
    for o in ops:
        flat.extend(_expand_rot(o) if o.name == "Rot" else [o])
    final = oracle.run(n, _oracle_ops(flat))
    obs = [(False, [(1.0, [("PauliZ", [2], None)])]),
           (True, [(0.4, [("PauliZ", [0], None), ("PauliZ", [1], None)]), (-1.2, [("PauliX", [3], None)]),
                   (0.7, [("PauliY", [2], None), ("PauliZ", [4], None)])])]
    ref = oracle.adjoint_jacobian(final, _oracle_ops(flat), obs, list(range(len(params))))
    assert np.max(np.abs(jac - ref)) < 1e-10


def test_vjp(oracle):
    rng = np.random.default_rng(3)
    n = 4
    ops = [Q.op("RY", w, rng.uniform(0, 6)) for w in range(n)] + [Q.op("CZ", [0, 1]), Q.op("RZ", 1, 0.3)]
    meas = [Q.expval(Q.PauliZ(0)), Q.expval(Q.PauliX(1) @ Q.PauliY(2))]
    tape = Q.QuantumTape(ops, meas)
    dev = _dev(n)
    dy = np.array([0.7, -1.3])
    v = dev.vjp(meas, dy)(tape)
    jac = dev.adjoint_jacobian(tape)
    assert np.allclose(v, dy @ jac, atol=1e-10)


def test_adjoint_rejects_unsupported():
    from pennylane_lightning_gpu_gb300.lightning_gpu import QuantumFunctionError

    dev = _dev(2)
    tape = Q.QuantumTape([Q.op("RX", 0, 0.1)], [Q.var(Q.PauliZ(0))])
    with pytest.raises(QuantumFunctionError):
        dev.adjoint_jacobian(tape)
    tape = Q.QuantumTape([Q.op("RX", 0, 0.1)], [Q.expval(Q.Hermitian(np.eye(2), [0]))])
    with pytest.raises(QuantumFunctionError):
        dev.adjoint_jacobian(tape)


def _central_differences(dev, ops, measurements, h=1e-4):
    params = [p for o in ops for p in o.parameters]

    def f(ps):
        k, new = 0, []
        for o in ops:
            m = len(o.parameters)
            base = Q.Operation(o.name, o.wires, ps[k:k + m], o._matrix)
            new.append(base.adjoint() if isinstance(o, Q.Adjoint) else base)
            k += m
        return np.array(dev.execute(Q.QuantumTape(new, measurements)))

    cols = []
    for i in range(len(params)):
        e = np.zeros(len(params))
        e[i] = h
        cols.append((f(np.array(params) + e) - f(np.array(params) - e)) / (2 * h))
    return np.stack(cols, axis=1)


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-10), (np.complex64, 1e-5)])
def test_adjoint_hermitian_opt_in(oracle, dtype, tol):
    """With adjoint_hermitian=True the adjoint Jacobian of Hermitian
    observables (alone, inside a tensor product and as a Hamiltonian term)
    matches the oracle's adjoint; the default keeps the reference's refusal."""
    from pennylane_lightning_gpu_gb300.lightning_gpu import QuantumFunctionError

    rng = np.random.default_rng(21)
    n = 5
    ops = [Q.op("RY", w, rng.uniform(0, 6)) for w in range(n)]
    ops += [Q.op("CNOT", [0, 1]), Q.op("CRX", [2, 4], 0.6), Q.op("RZ", 3, -0.9), Q.op("IsingXX", [1, 3], 0.4)]
    h2 = rng.normal(size=(4, 4)) + 1j * rng.normal(size=(4, 4))
    h2 = h2 + h2.conj().T
    h1 = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
    h1 = h1 + h1.conj().T
    H = Q.Hamiltonian([0.5, -0.7], [Q.Hermitian(h1, [2]), Q.PauliX(0) @ Q.PauliZ(4)])
    meas = [Q.expval(Q.Hermitian(h2, [3, 1])), Q.expval(Q.Hermitian(h1, [0]) @ Q.PauliY(4)), Q.expval(H)]
    tape = Q.QuantumTape(ops, meas)
    with pytest.raises(QuantumFunctionError):
        _dev(n, dtype).adjoint_jacobian(tape)
    dev = _dev(n, dtype, adjoint_hermitian=True)
    jac = dev.adjoint_jacobian(tape)
    final = oracle.run(n, _oracle_ops(ops))
    obs = [(False, [(1.0, [("Hermitian", [3, 1], h2)])]),
           (False, [(1.0, [("Hermitian", [0], h1), ("PauliY", [4], None)])]),
           (True, [(0.5, [("Hermitian", [2], h1)]), (-0.7, [("PauliX", [0], None), ("PauliZ", [4], None)])])]
    ntrain = sum(len(o.parameters) for o in ops)
    ref = oracle.adjoint_jacobian(final, _oracle_ops(ops), obs, list(range(ntrain)))
    scale = max(1.0, np.max(np.abs(ref)))
    assert np.max(np.abs(jac - ref)) < tol * 10 * scale
    # the vjp takes the same opt-in
    dy = np.array([0.3, -1.1, 0.8])
    v = dev.vjp(meas, dy)(tape)
    assert np.max(np.abs(v - dy @ ref)) < tol * 30 * scale


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-10), (np.complex64, 1e-5)])
def test_adjoint_multi_parameter_gates(oracle, dtype, tol):
    """CRot and inverted Rot/CRot (the reference's adjoint refuses them) through
    their one-parameter expansion: all parameters and a trainable subset that
    splits an inverted block, against the oracle adjoint on the expanded ops
    and (complex128) central differences."""
    from pennylane_lightning_gpu_gb300._serialize import _expand_rot, _expanded_param_positions

    rng = np.random.default_rng(23)
    n = 4
    ops = [Q.op("RY", w, rng.uniform(0, 6)) for w in range(n)]
    ops += [Q.op("CRot", [0, 2], 0.4, -1.3, 0.8), Q.op("Rot", 1, 1.1, 0.2, -0.6).adjoint(),
            Q.op("CNOT", [2, 3]), Q.op("CRot", [3, 1], -0.7, 2.1, 0.35).adjoint(), Q.op("Rot", 3, 0.5, 0.9, 1.7)]
    meas = [Q.expval(Q.PauliZ(1)), Q.expval(Q.PauliX(2) @ Q.PauliY(3))]
    nparams = sum(len(o.parameters) for o in ops)
    flat = []
    for o in ops:
        flat.extend(_expand_rot(o) if o.name in ("Rot", "CRot") else [o])
    final = oracle.run(n, _oracle_ops(flat))
    obs = [(False, [(1.0, [("PauliZ", [1], None)])]),
           (False, [(1.0, [("PauliX", [2], None), ("PauliY", [3], None)])])]
    ref_all = oracle.adjoint_jacobian(final, _oracle_ops(flat), obs, list(range(nparams)))
    pos = _expanded_param_positions(Q.QuantumTape(ops, meas))
    ref = ref_all[:, pos]  # columns back in tape order
    dev = _dev(n, dtype)
    for trainable in (list(range(nparams)), [1, 5, 7, 9, 12, 15]):
        tape = Q.QuantumTape(ops, meas, trainable)
        jac = dev.adjoint_jacobian(tape)
        assert jac.shape == (2, len(trainable))
        assert np.max(np.abs(jac - ref[:, trainable])) < tol * 10, trainable
    if dtype == np.complex128:
        fd = _central_differences(dev, ops, meas)
        assert np.max(np.abs(dev.adjoint_jacobian(Q.QuantumTape(ops, meas)) - fd)) < 1e-7


def test_adjoint_sparse_hamiltonian_vs_central_differences():
    """A SparseHamiltonian observable (CSR over all wires) in the adjoint
    Jacobian agrees with central differences of the device's own expectation
    (h = 1e-4, 1e-7)."""
    import scipy.sparse as sp

    rng = np.random.default_rng(22)
    n = 6
    dim = 1 << n
    a = sp.random(dim, dim, density=0.05, random_state=np.random.RandomState(3), format="csr",
                  dtype=np.float64)
    a = a + 1j * sp.random(dim, dim, density=0.05, random_state=np.random.RandomState(4), format="csr")
    herm = (a + a.conj().T).tocsr()
    ops = [Q.op("RX", w, rng.uniform(0, 6)) for w in range(n)]
    ops += [Q.op("CNOT", [0, 3]), Q.op("RY", 2, 0.3), Q.op("IsingZZ", [4, 5], 1.1), Q.op("CRZ", [1, 2], -0.5)]
    meas = [Q.expval(Q.SparseHamiltonian(herm, list(range(n)))), Q.expval(Q.PauliZ(2))]
    tape = Q.QuantumTape(ops, meas)
    dev = _dev(n)
    jac = dev.adjoint_jacobian(tape)
    fd = _central_differences(dev, ops, meas)
    assert np.max(np.abs(jac - fd)) < 1e-7


def test_mpi_rejected():
    from pennylane_lightning_gpu_gb300.lightning_gpu import DeviceError

    with pytest.raises(DeviceError):
        _dev(2, mpi=True)


@pytest.mark.parametrize("name,nw,n", [("QFT", 3, 5), ("QFT", 9, 11), ("GroverOperator", 4, 6),
                                       ("GroverOperator", 12, 13)])
def test_qft_and_grover_matrix_operations(oracle, name, nw, n):
    """QFT (below 10 wires) and GroverOperator (below 13) are applied as dense
    matrices, as the reference's stopping condition allows
    (lightning_gpu.py:504-511); wider ones raise."""
    rng = np.random.default_rng(nw)
    wires = [int(x) for x in rng.choice(n, size=nw, replace=False)]
    pre = [Q.op("Hadamard", w) for w in range(n)] + [Q.op("RY", w, 0.3 * (w + 1)) for w in range(n)]
    op = getattr(Q, name)(wires)
    dev = _dev(n)
    assert dev.supports_operation(op)
    dev.apply(pre + [op, op.adjoint() if name == "QFT" else Q.op("PauliX", wires[0])])
    tail = (op.matrix().conj().T, wires) if name == "QFT" else (np.array([[0, 1], [1, 0]]), [wires[0]])
    ref = oracle.run(n, _oracle_ops(pre) + [("QubitUnitary", wires, [], False, op.matrix()),
                                            ("QubitUnitary", tail[1], [], False, tail[0])])
    assert np.max(np.abs(dev.state - ref)) < 1e-10


def test_wide_qft_and_grover_are_refused():
    from pennylane_lightning_gpu_gb300.lightning_gpu import DeviceError

    dev = _dev(14)
    for op in (Q.QFT(list(range(10))), Q.GroverOperator(list(range(13)))):
        assert not dev.supports_operation(op)
        with pytest.raises(DeviceError, match="decompose"):
            dev.apply([op])

"""Batched persistent executor against the oracle and the plain per-circuit loop.

Tolerance: complex128 1e-10, complex64 1e-5 (absolute, per circuit result).
"""
import numpy as np
import pytest

from pennylane_lightning_gpu_gb300 import batched, workloads

pytestmark = pytest.mark.gpu


def _oracle_value(oracle, n, ops, obs):
    psi = oracle.run(n, [(o[0], o[1], o[2], o[3], None) for o in ops])
    words = [t[1] for t in obs]
    wires = [t[2] for t in obs]
    return oracle.expval_pauli_words(psi, words, wires, np.array([t[0] for t in obs], np.complex128))


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-10), (np.complex64, 1e-5)])
def test_batched_matches_oracle_small_and_large(oracle, dtype, tol):
    rng = np.random.default_rng(11)
    circuits = []
    for n in [3, 6, 10, 13, 14, 15, 16]:
        ops = workloads.random_circuit(n, 3, rng)
        ops += [("IsingXX", [0, n - 1], [0.4], False), ("SWAP", [1, n - 1], [], False),
                ("Toffoli", [0, 1, 2], [], False), ("PhaseShift", [n - 1], [0.7], True),
                ("CRX", [2, 0], [1.1], True), ("Hadamard", [n // 2], [], False), ("S", [1], [], True)]
        obs = workloads.random_pauli_hamiltonian(n, 6, rng, max_wires=3) + [(0.5, "Z", [n - 1])]
        circuits.append((n, ops, obs))
    ex = batched.build_executor(circuits, dtype)
    got = ex.run()
    for (n, ops, obs), g in zip(circuits, got):
        assert abs(g - _oracle_value(oracle, n, ops, obs)) < tol * 10, n


@pytest.mark.parametrize("dtype,tol", [(np.complex128, 1e-10), (np.complex64, 1e-5)])
def test_batched_param_replay(oracle, dtype, tol):
    circuits = batched.config2_circuits(count=24, nmin=8, nmax=15, seed=5)
    ex = batched.build_executor(circuits, dtype)
    first = ex.run()
    ref_plain = batched.plain_loop(circuits, dtype)
    assert np.max(np.abs(first - ref_plain)) < tol * 100
    # new parameters through the captured graph
    p = ex.params
    rng = np.random.default_rng(1)
    newp = rng.uniform(0, 2 * np.pi, p.size)
    got = ex.run(newp)
    k = 0
    for ci, (n, ops, obs) in enumerate(circuits):
        new_ops = []
        for o in ops:
            if o[2]:
                new_ops.append((o[0], o[1], [float(newp[k])], o[3]))
                k += 1
            else:
                new_ops.append(o)
        assert abs(got[ci] - _oracle_value(oracle, n, new_ops, obs)) < tol * 10


def test_batched_config2_subset_vs_plain():
    circuits = batched.config2_circuits(count=64, seed=2)
    ex = batched.build_executor(circuits, np.complex128)
    got = ex.run()
    ref = batched.plain_loop(circuits, np.complex128, fusion=True)
    assert np.max(np.abs(got - ref)) < 1e-9


def test_autotune_cache(tmp_path, monkeypatch):
    monkeypatch.setenv("LGPU_AUTOTUNE_CACHE", str(tmp_path / "tune.json"))
    circuits = batched.config2_circuits(count=32, nmin=10, nmax=14, seed=3)
    k, t, rec = batched.autotune(circuits, np.complex64, sample=16, repeats=1,
                                 candidates=[(12, 256), (14, 256)])
    assert (k, t) in [(12, 256), (14, 256)]
    k2, t2, rec2 = batched.autotune(circuits, np.complex64, sample=16, repeats=1)
    assert (k2, t2) == (k, t)


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_templates_match_per_circuit_adds(dtype):
    """The same batch added as templates plus parameter rows and as one
    circuit at a time gives the same bits per circuit."""
    templates, order = batched.config2_templates(count=200, nmin=10, nmax=18, seed=7)
    circuits = batched.config2_circuits(count=200, nmin=10, nmax=18, seed=7)
    a = batched.build_executor(circuits, dtype).run()
    ex = batched.build_executor_from_templates(templates, dtype, capture=False)
    b = ex.run()
    base = np.cumsum([0] + [p.shape[0] for _, p in templates])
    got = np.array([b[base[ti] + row] for ti, row in order])
    assert np.array_equal(got, a)


def test_add_reads_op_tuples_of_any_numeric_type(oracle):
    """add() hands the op tuples to the native side as they are: numpy wires
    and parameters, ops without the inverse flag, numpy booleans and tuples
    instead of lists give the same circuit; a malformed op raises."""
    n = 9
    rng = np.random.default_rng(3)
    ops = workloads.random_circuit(n, 2, rng) + [("PhaseShift", [4], [0.3], True), ("CRX", [2, 5], [0.9], True)]
    obs = workloads.random_pauli_hamiltonian(n, 5, rng, max_wires=3)
    odd_ops = []
    for i, (name, wires, params, inv) in enumerate(ops):
        if i % 2 == 0 and not inv:
            odd_ops.append((name, np.array(wires, np.int64), np.array(params, np.float64)))
        else:
            odd_ops.append((name, tuple(wires), tuple(np.float64(x) for x in params), np.bool_(inv)))
    odd_obs = [(np.float64(c), w, np.array(ws)) for c, w, ws in obs]
    ex = batched.BatchedExecutor(np.complex128)
    ex.add(n, ops, obs)
    ex.add(n, odd_ops, odd_obs)
    ex.prepare(capture=False)
    a, b = ex.run()
    assert abs(a - _oracle_value(oracle, n, ops, obs)) < 1e-10
    assert a == b
    bad = batched.BatchedExecutor(np.complex128)
    with pytest.raises(Exception):
        bad.add(n, [("RX", [0])], obs)

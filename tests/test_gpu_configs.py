"""Parity at the benchmarked configurations, against the FP64 oracle.

Each case builds its input with the same generator and seed as the bench
(``workloads.circuit_28q_workload``, ``workloads.adjoint_24q_workload``,
``batched.config2_circuits``, ``workloads.layered_ansatz``) and compares the
engine's result with the oracle's on the same input.

Tolerances (absolute):
  * states and single expectation values: complex128 1e-10, complex64 1e-5;
  * a weighted sum of Pauli words sum_j c_j <P_j>: the same bound times
    max(1, sum_j |c_j|) (each <P_j> carries its own error);
  * Jacobians: the same scaled bound;
  * central differences (h = 1e-4) of a sum of Pauli rotations' expectation:
    h^2 / 6 * sum_j |c_j| (the truncation bound: every parameter enters as
    a + b cos(theta) + c sin(theta) with |b| + |c| <= sum_j |c_j|) + 1e-9 for rounding;
  * sampling: indices bit-exact with the oracle's sampler run on the state the
    device holds, with the same seeded draws.
"""
import numpy as np
import pytest

from pennylane_lightning_gpu_gb300 import batched, workloads
from pennylane_lightning_gpu_gb300 import ops as Q

pytestmark = pytest.mark.gpu

TOL = {np.complex128: 1e-10, np.complex64: 1e-5}


def _dev(n, dtype):
    from pennylane_lightning_gpu_gb300.lightning_gpu import LightningGPU

    return LightningGPU(n, c_dtype=dtype)


def _oracle_obs(terms):
    return (True, [(c, [("Pauli" + ch, [w], None) for ch, w in zip(word, wires)]) for c, word, wires in terms])


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_layered_12q_jacobian_exact_config(oracle, dtype):
    """12 qubits, 4 layers of RX, RY, RZ on every wire + CNOT ring (seed 0):
    the 12 <Z_i> and the 12 x 144 adjoint Jacobian through the device."""
    n, layers = 12, 4
    raw = workloads.layered_ansatz(n, layers, np.random.default_rng(0))
    ops = [Q.op(o[0], o[1], *o[2]) for o in raw]
    tape = Q.QuantumTape(ops, [Q.expval(Q.PauliZ(w)) for w in range(n)])
    dev = _dev(n, dtype)
    vals = np.asarray(dev.execute(tape))
    jac = np.asarray(dev.adjoint_jacobian(tape))
    oops = [(o[0], o[1], o[2], False, None) for o in raw]
    psi = oracle.run(n, oops)
    z = np.diag([1.0, -1.0])
    ref_vals = np.array([oracle.expval_matrix(psi, z, [w]).real for w in range(n)])
    obs = [(False, [(1.0, [("PauliZ", [w], None)])]) for w in range(n)]
    nparams = sum(1 for o in raw if o[2])
    ref_jac = oracle.adjoint_jacobian(psi, oops, obs, list(range(nparams)))
    assert jac.shape == (n, 3 * n * layers)
    assert np.max(np.abs(vals - ref_vals)) < TOL[dtype]
    assert np.max(np.abs(jac - ref_jac)) < TOL[dtype]


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
@pytest.mark.parametrize("n", [20, 24])
def test_840_gate_circuit_vs_oracle(oracle, dtype, n):
    """The 28-qubit circuit generator at n = 20 and 24 with all 840 operations
    (20 layers of 28 rotations + 14 CNOT/CZ/CRY) through the fused path
    (complex128 runs these blocks in float-float arithmetic): the state, the
    100-term Hamiltonian, probabilities on 10 wires and 1e4 seeded shots."""
    raw, terms = workloads.circuit_28q_workload(n)
    assert len(raw) == 840
    ops = [Q.op(o[0], o[1], *o[2]) for o in raw]
    dev = _dev(n, dtype)
    dev.apply(ops)
    got = dev.state.astype(np.complex128)
    psi = oracle.run(n, [(o[0], o[1], o[2], False, None) for o in raw])
    tol = TOL[dtype]
    assert np.max(np.abs(got - psi)) < tol

    from pennylane_lightning_gpu_gb300 import torch_adjoint as TA

    H = TA.pauli_hamiltonian(terms)
    scale = max(1.0, sum(abs(t[0]) for t in terms))
    e = dev.expval(H)
    e_ref = oracle.expval_pauli_words(psi, [t[1] for t in terms], [t[2] for t in terms],
                                      np.array([t[0] for t in terms], np.complex128))
    assert abs(e - e_ref) < tol * scale, (e, e_ref)

    wires = list(range(10))
    p = np.asarray(dev.probability(wires=wires))
    p_ref = oracle.probs(psi, wires).reshape([2] * 10).transpose().reshape(-1)  # PennyLane order
    assert np.max(np.abs(p - p_ref)) < tol

    seed, shots = 77, 10000
    dev._gpu_state.setSeed(seed)
    idx = np.asarray(dev._gpu_state.GenerateSampleIndices(shots, True))
    held = dev.state.astype(np.complex128)
    ref_idx = oracle.sample_indices(held, seed, shots, float_draws=(dtype == np.complex64))
    assert int(np.sum(idx != ref_idx)) == 0


def test_adjoint_24q_384_params_vs_oracle_and_fd(oracle):
    """24 qubits, 8 layers of RY, RZ + CZ ladder (384 parameters), 50-term
    Hamiltonian, through torch.autograd: every Jacobian column against the
    oracle adjoint, and 8 seeded columns against central differences."""
    torch = pytest.importorskip("torch")
    from pennylane_lightning_gpu_gb300 import torch_adjoint as TA

    n, layers = 24, 8
    terms, params = workloads.adjoint_24q_workload(n, layers)
    H = TA.pauli_hamiltonian(terms)
    template = TA.ry_rz_cz_template(n, layers)
    dev = _dev(n, np.complex128)
    f = TA.expval_function(template, [H], dev)
    p = torch.tensor(params, dtype=torch.float64, requires_grad=True)
    y = f(p)
    y.sum().backward()
    grad = p.grad.numpy()
    assert grad.shape == (384,)

    ops = template(params)
    oops = [(o.name, o.wires, o.parameters, False, None) for o in ops]
    assert len(oops) == 568
    final = oracle.run(n, oops)
    ref = oracle.adjoint_jacobian(final, oops, [_oracle_obs(terms)], list(range(params.size)))[0]
    scale = max(1.0, sum(abs(t[0]) for t in terms))
    assert np.max(np.abs(grad - ref)) < 1e-10 * scale
    e_ref = oracle.expval_pauli_words(final, [t[1] for t in terms], [t[2] for t in terms],
                                      np.array([t[0] for t in terms], np.complex128))
    assert abs(float(y.detach()[0]) - e_ref) < 1e-10 * scale

    cols = sorted(np.random.default_rng(3).choice(params.size, size=8, replace=False).tolist())
    h = 1e-4
    fd = TA.central_differences(template, [H], dev, params, h=h, indices=cols)[0]
    assert np.max(np.abs(grad[cols] - fd)) < h * h / 6 * scale + 1e-9


@pytest.mark.parametrize("dtype", [np.complex128, np.complex64])
def test_batched_4096_circuits_vs_oracle(oracle, dtype):
    """The 4096-circuit batch (10..20 qubits, seed 2) in one persistent
    launch; every circuit of 17..20 qubits in a seeded sample of 24 against
    the oracle's sum_i <Z_i>."""
    circuits = batched.config2_circuits(count=4096, seed=2)
    ex = batched.build_executor(circuits, dtype)
    got = ex.run()
    rng = np.random.default_rng(21)
    big = [i for i, c in enumerate(circuits) if c[0] >= 17]
    pick = sorted(rng.choice(big, size=24, replace=False).tolist())
    worst = 0.0
    for i in pick:
        n, ops, obs = circuits[i]
        psi = oracle.run(n, [(o[0], o[1], o[2], o[3], None) for o in ops])
        ref = oracle.expval_pauli_words(psi, [t[1] for t in obs], [t[2] for t in obs],
                                        np.array([t[0] for t in obs], np.complex128))
        worst = max(worst, abs(got[i] - ref) / max(1.0, float(n)))
    assert worst < TOL[dtype]

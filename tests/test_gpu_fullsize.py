"""Size-independent properties at the benchmark's full size: 28 qubits
(complex128 4 GiB, complex64 2 GiB), where the oracle cannot follow.

* U then U^dag (the inverse circuit) returns |0...0> (the marginal of the
  first ten wires puts all weight on 0): complex128 1e-10, complex64 1e-4;
* the norm is preserved by 840 gates (marginals sum to 1);
* the fused multi-op path and the one-gate-per-launch path give the same
  marginals and Pauli expectations (complex128 1e-10, complex64 1e-5);
* Pauli-word sums are linear: <sum_t c_t P_t> = sum_t c_t <P_t>;
* 1e4 samples reproduce the one-wire marginal within 5 standard deviations.
"""
import numpy as np
import pytest

from pennylane_lightning_gpu_gb300 import workloads

pytestmark = pytest.mark.gpu

N = 28
TOLS = {"c128": 1e-10, "c64": 1e-5}


def _cls(native, dtype):
    return getattr(native, "LightningGPU_C128" if dtype == "c128" else "LightningGPU_C64")


def _apply(sv, ops, per_gate=False):
    if per_gate:
        for name, wires, params, inv in ops:
            sv.apply(name, list(wires), bool(inv), list(params), np.zeros(0))
    else:
        sv.apply([o[0] for o in ops], [list(o[1]) for o in ops], [bool(o[3]) for o in ops],
                 [list(o[2]) for o in ops])


def _inverse(ops):
    return [(name, wires, params, not inv) for name, wires, params, inv in reversed(ops)]


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_round_trip_returns_to_zero_state(native, dtype):
    ops = workloads.random_circuit(N, 20, np.random.default_rng(11))
    sv = _cls(native, dtype)(N)
    _apply(sv, ops)
    p = np.asarray(sv.Probability(list(range(10))))
    assert abs(p.sum() - 1.0) < (1e-10 if dtype == "c128" else 1e-4)
    assert p[0] < 0.5  # the circuit moved the state away from |0>
    _apply(sv, _inverse(ops))
    p = np.asarray(sv.Probability(list(range(10))))
    assert abs(p[0] - 1.0) < (1e-10 if dtype == "c128" else 1e-4), p[0]


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_fused_and_per_gate_paths_agree(native, dtype):
    ops = workloads.random_circuit(N, 3, np.random.default_rng(12))
    words = [t[1] for t in workloads.random_pauli_hamiltonian(N, 12, np.random.default_rng(13), max_wires=4)]
    wires = [list(t[2]) for t in workloads.random_pauli_hamiltonian(N, 12, np.random.default_rng(13), max_wires=4)]
    res = []
    for per_gate in (False, True):
        sv = _cls(native, dtype)(N)
        _apply(sv, ops, per_gate=per_gate)
        p = np.asarray(sv.Probability(list(range(N - 10, N))))
        ev = [float(sv.ExpectationValue([w], [ws], np.ones(1, np.complex128 if dtype == "c128" else np.complex64)))
              for w, ws in zip(words, wires)]
        res.append((p, np.array(ev)))
        del sv
    assert np.max(np.abs(res[0][0] - res[1][0])) < TOLS[dtype]
    assert np.max(np.abs(res[0][1] - res[1][1])) < TOLS[dtype] * 10


@pytest.mark.parametrize("dtype", ["c128", "c64"])
def test_pauli_sum_is_linear(native, dtype):
    ops = workloads.random_circuit(N, 2, np.random.default_rng(14))
    terms = workloads.random_pauli_hamiltonian(N, 40, np.random.default_rng(15), max_wires=6)
    cdt = np.complex128 if dtype == "c128" else np.complex64
    sv = _cls(native, dtype)(N)
    _apply(sv, ops)
    coeffs = np.array([t[0] for t in terms], cdt)
    total = float(sv.ExpectationValue([t[1] for t in terms], [list(t[2]) for t in terms], coeffs))
    single = [float(sv.ExpectationValue([t[1]], [list(t[2])], np.ones(1, cdt))) for t in terms]
    assert abs(total - float(np.dot(coeffs.real.astype(np.float64), single))) < TOLS[dtype] * 40


def test_samples_follow_marginal(native):
    ops = workloads.random_circuit(N, 2, np.random.default_rng(16))
    sv = native.LightningGPU_C128(N)
    _apply(sv, ops)
    p1 = float(np.asarray(sv.Probability([0]))[1])
    sv.setSeed(1234)
    shots = 10000
    samples = np.asarray(sv.GenerateSamples(N, shots))
    assert samples.shape == (shots, N)
    freq = samples[:, 0].mean()
    sigma = np.sqrt(p1 * (1 - p1) / shots)
    assert abs(freq - p1) < 5 * sigma + 1e-12

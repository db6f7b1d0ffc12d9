"""Edge cases through the pybind11 interface: the smallest states, empty
inputs and out-of-range sizes (complex128 1e-10, complex64 1e-5 against the
oracle where a value is compared)."""
import numpy as np
import pytest

from helpers import cls_name, make_sv, np_dtype, random_state, to_oracle_ops, tol

pytestmark = pytest.mark.gpu

DTYPES = ["c128", "c64"]
ONE_QUBIT = [("Identity", []), ("PauliX", []), ("PauliY", []), ("PauliZ", []), ("Hadamard", []), ("S", []),
             ("T", []), ("RX", [0.3]), ("RY", [1.2]), ("RZ", [2.5]), ("PhaseShift", [0.7]), ("Rot", [0.1, 0.2, 0.3])]


@pytest.mark.parametrize("dtype", DTYPES)
def test_one_qubit_state(native, oracle, dtype):
    rng = np.random.default_rng(1)
    psi = random_state(1, rng)
    ops = [(name, [0], params, bool(i % 2)) for i, (name, params) in enumerate(ONE_QUBIT)]
    sv = make_sv(native, dtype, psi)
    for o in ops:
        sv.apply(o[0], o[1], o[3], o[2], np.zeros(0, np_dtype(dtype)))
    ref = oracle.apply_ops(psi, to_oracle_ops(ops))
    assert np.max(np.abs(sv.GetState() - ref)) < tol(dtype)
    p = np.asarray(sv.Probability([0]))
    assert np.max(np.abs(p - np.abs(ref) ** 2)) < tol(dtype)
    z = float(sv.ExpectationValue(["Z"], [[0]], np.ones(1, np_dtype(dtype))))
    assert abs(z - (abs(ref[0]) ** 2 - abs(ref[1]) ** 2)) < tol(dtype)


@pytest.mark.parametrize("dtype", DTYPES)
def test_two_qubit_fused_list(native, oracle, dtype):
    rng = np.random.default_rng(2)
    psi = random_state(2, rng)
    ops = [("Hadamard", [0], [], False), ("CNOT", [0, 1], [], False), ("RY", [1], [0.4], True),
           ("CRZ", [1, 0], [1.1], False), ("SWAP", [0, 1], [], False), ("IsingZZ", [0, 1], [0.6], False)]
    sv = make_sv(native, dtype, psi)
    sv.apply([o[0] for o in ops], [o[1] for o in ops], [o[3] for o in ops], [o[2] for o in ops])
    ref = oracle.apply_ops(psi, to_oracle_ops(ops))
    assert np.max(np.abs(sv.GetState() - ref)) < tol(dtype)


@pytest.mark.parametrize("dtype", DTYPES)
def test_empty_inputs(native, dtype):
    rng = np.random.default_rng(3)
    psi = random_state(4, rng)
    sv = make_sv(native, dtype, psi)
    sv.apply([], [], [], [])  # no operations: state unchanged
    assert np.max(np.abs(sv.GetState() - psi)) < tol(dtype)
    v = float(sv.ExpectationValue([], [], np.zeros(0, np_dtype(dtype))))  # empty Pauli sum
    assert v == 0.0
    samples = np.asarray(sv.GenerateSamples(4, 0))
    assert samples.size == 0


@pytest.mark.parametrize("dtype", DTYPES)
def test_out_of_range_sizes_raise(native, dtype):
    cls = getattr(native, cls_name(dtype))
    with pytest.raises(Exception):
        cls(35)  # beyond the 34-qubit limit: rejected before any allocation
    sv = cls(3)
    with pytest.raises(Exception):
        sv.apply("RX", [3], False, [0.1], np.zeros(0, np_dtype(dtype)))  # wire out of range
    with pytest.raises(Exception):
        sv.Probability([0, 5])


def test_adjoint_needs_trainable_parameters(native):
    sv = native.LightningGPU_C128(2)
    adj = native.AdjointJacobianGPU_C128()
    opsd = adj.create_ops_list(["RX"], [np.array([0.1])], [[0]], [False], [np.zeros(0, np.complex128)])
    with pytest.raises(native.PLException, match="No trainable parameters"):
        adj.adjoint_jacobian(sv, [native.NamedObsGPU_C128("PauliZ", [0])], opsd, [])


@pytest.mark.parametrize("dtype", DTYPES)
def test_all_wire_probabilities_and_basis_states(native, dtype):
    for n in (1, 3):
        sv = getattr(native, cls_name(dtype))(n)
        for idx in range(1 << n):
            sv.setBasisState(idx, False)
            p = np.asarray(sv.Probability(list(range(n))))
            # Probability is LSB-first over the given wires (bit k <-> wires[k])
            want = np.zeros(1 << n)
            rev = int(format(idx, "0%db" % n)[::-1], 2)
            want[rev] = 1.0
            assert np.max(np.abs(p - want)) < tol(dtype), (n, idx, p)


@pytest.mark.parametrize("dtype", DTYPES)
def test_reductions_after_sampling_and_adjoint(native, oracle, dtype):
    """Scratch contexts are reused across calls and, through the library's
    free list, across states: sampling an unnormalised state (a total that is
    not 1) and a whole adjoint sweep must leave later reductions intact."""
    rng = np.random.default_rng(5)
    psi = 0.7 * random_state(6, rng)
    sv = make_sv(native, dtype, psi)
    sv.setSeed(3)
    idx = np.asarray(sv.GenerateSampleIndices(100, True))
    assert idx.size == 100
    p = np.asarray(sv.Probability([0, 1]))
    ref = oracle.probs(psi.astype(np.complex128), [0, 1])
    assert np.max(np.abs(p - ref)) < tol(dtype)
    # adjoint on a small state (whole sweep in one launch), then a fresh state
    a = getattr(native, cls_name(dtype))(4)
    a.apply(["RX", "CNOT", "RY"], [[0], [0, 1], [1]], [False] * 3, [[0.3], [], [0.8]])
    suf = "C128" if dtype == "c128" else "C64"
    adj = getattr(native, "AdjointJacobianGPU_" + suf)()
    rdt = np.float64 if dtype == "c128" else np.float32
    opsd = adj.create_ops_list(["RX", "CNOT", "RY"], [np.array([0.3], rdt), np.zeros(0, rdt), np.array([0.8], rdt)],
                               [[0], [0, 1], [1]], [False] * 3, [np.zeros(0, np_dtype(dtype))] * 3)
    adj.adjoint_jacobian(a, [getattr(native, "NamedObsGPU_" + suf)("PauliZ", [1])], opsd, [0, 1])
    del a
    for _ in range(3):
        b = make_sv(native, dtype, random_state(5, rng))
        st = np.asarray(b.GetState()).astype(np.complex128)
        z = float(b.ExpectationValue(["Z"], [[0]], np.ones(1, np_dtype(dtype))))
        want = float(np.sum(np.abs(st[:16]) ** 2) - np.sum(np.abs(st[16:]) ** 2))
        assert abs(z - want) < tol(dtype) * 10
        del b

"""GPU parity of the drop-in classes against the CPU oracle.

Tolerances (written per test): complex128 1e-10 absolute per amplitude /
expectation, complex64 1e-5, both against the FP64 oracle; sampling indices
bit-exact for the same seeded draw stream.
"""
import itertools
import zlib

import numpy as np
import pytest

from helpers import (apply_ops, cls_name, make_sv, np_dtype, random_hermitian, random_state, random_unitary,
                     to_oracle_ops, tol)

pytestmark = pytest.mark.gpu

DTYPES = ["c128", "c64"]

# (name, number of wires, number of params)
GATES = [
    ("Identity", 1, 0), ("PauliX", 1, 0), ("PauliY", 1, 0), ("PauliZ", 1, 0), ("Hadamard", 1, 0), ("S", 1, 0),
    ("T", 1, 0), ("RX", 1, 1), ("RY", 1, 1), ("RZ", 1, 1), ("PhaseShift", 1, 1), ("Rot", 1, 3),
    ("CNOT", 2, 0), ("CY", 2, 0), ("CZ", 2, 0), ("SWAP", 2, 0), ("CRX", 2, 1), ("CRY", 2, 1), ("CRZ", 2, 1),
    ("CRot", 2, 3), ("ControlledPhaseShift", 2, 1), ("IsingXX", 2, 1), ("IsingYY", 2, 1), ("IsingZZ", 2, 1),
    ("SingleExcitation", 2, 1), ("SingleExcitationMinus", 2, 1), ("SingleExcitationPlus", 2, 1),
    ("CSWAP", 3, 0), ("Toffoli", 3, 0), ("DoubleExcitation", 4, 1), ("DoubleExcitationMinus", 4, 1),
    ("DoubleExcitationPlus", 4, 1), ("MultiRZ", 1, 1), ("MultiRZ", 3, 1), ("MultiRZ", 5, 1),
]


def _check(native, oracle, dtype, n, ops, rng, per_gate=False):
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    if per_gate:
        for o in ops:
            getattr(sv, o[0])(list(o[1]), bool(o[3]), list(o[2]))
    else:
        apply_ops(sv, ops)
    got = sv.GetState()
    ref = oracle.apply_ops(psi, to_oracle_ops(ops))
    err = np.max(np.abs(got - ref))
    assert err < tol(dtype), (ops, err)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [5, 7])
@pytest.mark.parametrize("name,nw,npar", GATES)
def test_named_gate(native, oracle, dtype, n, name, nw, npar):
    rng = np.random.default_rng(zlib.crc32(('%s-%d-%d-%s' % (name, nw, n, dtype)).encode()))
    for trial in range(4):
        wires = [int(x) for x in rng.choice(n, size=nw, replace=False)]
        params = [float(x) for x in rng.uniform(0, 2 * np.pi, npar)]
        for adj in (False, True):
            _check(native, oracle, dtype, n, [(name, wires, params, adj)], rng)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("name,nw,npar", [g for g in GATES if g[0] != "Identity"])
def test_per_gate_methods(native, oracle, dtype, name, nw, npar):
    rng = np.random.default_rng(7 + nw)
    n = 6
    for _ in range(3):
        wires = [int(x) for x in rng.choice(n, size=nw, replace=False)]
        params = [float(x) for x in rng.uniform(0, 2 * np.pi, npar)]
        for adj in (False, True):
            _check(native, oracle, dtype, n, [(name, wires, params, adj)], rng, per_gate=True)


@pytest.mark.parametrize("dtype", DTYPES)
def test_controlled_per_gate_semantics(native, oracle, dtype):
    """Per-gate methods take wires[:-1] as controls (PauliX on 3 wires = Toffoli)."""
    rng = np.random.default_rng(3)
    n = 5
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    sv.PauliX([0, 3, 1], False, [])
    sv.RY([4, 2], True, [0.7])
    ref = oracle.apply_ops(psi, [("Toffoli", [0, 3, 1], [], False, None), ("CRY", [4, 2], [0.7], True, None)])
    assert np.max(np.abs(sv.GetState() - ref)) < tol(dtype)


def _wide_unitary(t, rng):
    """A dense 2^t x 2^t unitary without a 2^t-sized QR: random phases times
    the Kronecker product of random unitaries on at most 3 wires each, with
    its rows permuted (every entry is generally non-zero)."""
    u = np.ones((1, 1), complex)
    left = t
    while left:
        k = min(3, left)
        u = np.kron(u, random_unitary(1 << k, rng))
        left -= k
    d = 1 << t
    return (np.exp(2j * np.pi * rng.random(d))[:, None] * u)[rng.permutation(d)]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("t", [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12])
def test_dense_matrix(native, oracle, dtype, t):
    """Dense QubitUnitary on t = 1..12 targets (12 is the reference's widest
    dense matrix gate: GroverOperator below 13 wires)."""
    rng = np.random.default_rng(100 + t)
    n = max(t + 2, 6)
    for adj in (False, True):
        u = random_unitary(1 << t, rng) if t <= 7 else _wide_unitary(t, rng)
        wires = [int(x) for x in rng.choice(n, size=t, replace=False)]
        _check(native, oracle, dtype, n, [("QubitUnitary", wires, [], adj, u)], rng)


@pytest.mark.parametrize("dtype", DTYPES)
def test_unsupported_gate_raises(native, dtype):
    sv = getattr(native, cls_name(dtype))(3)
    with pytest.raises(native.PLException, match="Currently unsupported gate: NoSuchGate"):
        sv.apply("NoSuchGate", [0], False, [], np.zeros(0))


@pytest.mark.parametrize("dtype", DTYPES)
def test_bad_wire_raises(native, dtype):
    sv = getattr(native, cls_name(dtype))(3)
    with pytest.raises(native.PLException):
        sv.RX([5], False, [0.1])


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n,layers", [(6, 3), (9, 4), (12, 3), (13, 2)])
def test_fused_random_circuit(native, oracle, dtype, n, layers):
    from pennylane_lightning_gpu_gb300 import workloads

    rng = np.random.default_rng(n * 31 + layers)
    ops = workloads.random_circuit(n, layers, rng)
    ops += [("IsingXX", [0, n - 1], [0.3], False), ("SWAP", [1, 2], [], False), ("Toffoli", [0, 1, 2], [], False),
            ("S", [n - 2], [], True), ("MultiRZ", list(range(min(n, 5))), [0.9], False)]
    psi = random_state(n, rng)
    for fusion in (True, False):
        sv = make_sv(native, dtype, psi)
        sv.setFusion(fusion)
        sv.apply([o[0] for o in ops], [o[1] for o in ops], [o[3] for o in ops], [o[2] for o in ops])
        ref = oracle.apply_ops(psi, to_oracle_ops(ops))
        err = np.max(np.abs(sv.GetState() - ref))
        assert err < tol(dtype) * (10 if dtype == "c64" else 1), (fusion, err)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("k", [1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13])
def test_expval_matrix(native, oracle, dtype, k):
    """<psi|H|psi> for a dense Hermitian H on k = 1..13 wires (13: the widest
    Hamiltonian the reference's device hands over as one dense matrix)."""
    rng = np.random.default_rng(200 + k)
    n = k + 3 if k <= 7 else k + 1
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    h = random_hermitian(1 << k, rng)
    if k > 7:
        h /= np.sqrt(1 << k)  # spectral norm O(1)
    wires = [int(x) for x in rng.choice(n, size=k, replace=False)]
    got = sv.ExpectationValue(wires, h.ravel())
    ref = oracle.expval_matrix(psi, h, wires).real
    assert abs(got - ref) < tol(dtype) * max(1.0, np.abs(h).max()) * 10
    got2 = sv.ExpectationValue("Hermitian_%d" % k, wires, [], h.ravel())
    assert abs(got2 - ref) < tol(dtype) * max(1.0, np.abs(h).max()) * 10


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("k", [1, 2, 3])
def test_expval_matrix_float_float_paths(native, oracle, dtype, k):
    """1- and 2-target expectations go through Gram sums (G_rc = sum conj(a_r)
    a_c, contracted with M at the end), 3-target ones through conj(a).(M a)
    per group in float-float: Hermitian and general complex matrices, both
    parts of the complex result (through the C ABI), targets low, high and
    mixed, on a 20-qubit state so that many CTAs take part."""
    import ctypes

    import pennylane_lightning_gpu_gb300 as pkg

    rng = np.random.default_rng(250 + k)
    n = 20
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    lib = ctypes.CDLL(pkg.library_path())
    dp = ctypes.POINTER(ctypes.c_double)
    ctx = ctypes.c_void_p()
    assert lib.lgpu_context_create(0, ctypes.byref(ctx)) == 0
    try:
        for wires in (list(range(k)), list(range(n - k, n)), [int(x) for x in rng.choice(n, k, replace=False)]):
            for m in (random_hermitian(1 << k, rng), random_unitary(1 << k, rng)):
                ref = oracle.expval_matrix(psi, m, wires)
                got = sv.ExpectationValue(wires, m.ravel())
                assert abs(got - ref.real) < tol(dtype) * 10, (wires, got, ref)
                # both parts through the C ABI (targets as state bits, first = most significant matrix bit)
                mat = np.ascontiguousarray(m, np.complex128).view(np.float64)
                bits = np.array([n - 1 - w for w in wires], np.int32)
                out = np.zeros(2)
                rc = lib.lgpu_expval_matrix(ctx, ctypes.c_void_p(sv.dataPtr()), ctypes.c_uint32(n),
                                            ctypes.c_int(1 if dtype == "c128" else 0), mat.ctypes.data_as(dp),
                                            ctypes.c_uint32(k), bits.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                            out.ctypes.data_as(dp), ctypes.c_int(0), ctypes.c_void_p(sv.streamPtr()))
                assert rc == 0
                assert abs(complex(out[0], out[1]) - ref) < tol(dtype) * 10, (wires, out, ref)
    finally:
        lib.lgpu_context_destroy(ctx)

    rng = np.random.default_rng(11)
    n = 6
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    mats = {"PauliX": np.array([[0, 1], [1, 0]]), "PauliY": np.array([[0, -1j], [1j, 0]]),
            "PauliZ": np.diag([1, -1]), "Hadamard": np.array([[1, 1], [1, -1]]) / np.sqrt(2)}
    for name, m in mats.items():
        for w in range(n):
            got = sv.ExpectationValue(name, [w], [], np.zeros(0, np.complex128))
            ref = oracle.expval_matrix(psi, m, [w]).real
            assert abs(got - ref) < tol(dtype)
    # tensor observable via the vector-of-names overload
    m = np.kron(mats["PauliX"], mats["PauliZ"])
    got = sv.ExpectationValue(["PauliX", "PauliZ"], [4, 1], [[], []], m.ravel())
    assert abs(got - oracle.expval_matrix(psi, m, [4, 1]).real) < tol(dtype)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [4, 9, 14, 16, 18])
def test_pauli_words(native, oracle, dtype, n):
    """Pauli-word sums and single words against the oracle.  From 16 qubits
    words with different flip masks share tile passes; words flipping more
    bits than a tile holds (the 8- and 9-letter X/Y words) take the flip-mask
    passes in the same call."""
    from pennylane_lightning_gpu_gb300 import workloads

    rng = np.random.default_rng(300 + n)
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    ham = workloads.random_pauli_hamiltonian(n, 40, rng, max_wires=min(6, n))
    ham += [(0.5, "ZZ", [0, 1]), (-0.25, "ZZ", [1, 2]), (0.1, "XX", [0, 1]), (0.2, "XX", [0, 1]), (0.3, "I", [0])]
    if n >= 9:
        ham += [(0.4, "XYXYXYXY", list(range(8))), (-0.3, "YYXXZXYXY", list(range(n - 9, n)))]
    words = [h[1] for h in ham]
    wires = [h[2] for h in ham]
    coeffs = np.array([h[0] for h in ham], np.complex128)
    got = sv.ExpectationValue(words, wires, coeffs.astype(np_dtype(dtype)))
    ref = oracle.expval_pauli_words(psi, words, wires, coeffs)
    assert abs(got - ref) < tol(dtype) * len(ham)
    per = sv.PauliWordExpectations(words, wires)
    for j, h in enumerate(ham):
        rj = oracle.expval_pauli_words(psi, [h[1]], [h[2]], np.array([1.0]))
        assert abs(per[j] - rj) < tol(dtype), (h, per[j], rj)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("nwords", [3, 12, 30])
def test_pauli_tile_pass_counts(native, oracle, dtype, nwords):
    """Tile passes on an 18-qubit state with one, a few and many passes
    (complex128 converts each tile in the pass itself below three passes and
    reads a float-float copy of the state from three on): every word against
    the oracle.  The words mix diagonal ones, real and imaginary pair sums,
    flips on bit 0, on the bits of a tile's per-thread index part (8..10) and
    on the highest state bits."""
    n = 18
    rng = np.random.default_rng(77 + nwords)
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    fixed = [("Z", [0]), ("ZZZ", [3, 9, 17]), ("X", [n - 1]), ("XY", [n - 1, n - 2]), ("YX", [n - 9, n - 10]),
             ("XZY", [n - 1, n - 5, n - 11]), ("XXYYX", [0, 4, 8, 12, 16]), ("Y", [n - 3])]
    words = [w for w, _ in fixed][:nwords]
    wires = [ws for _, ws in fixed][:nwords]
    while len(words) < nwords:
        k = int(rng.integers(1, 7))
        ws = [int(x) for x in rng.choice(n, size=k, replace=False)]
        words.append("".join(rng.choice(list("XYZ"), size=k)))
        wires.append(ws)
    per = sv.PauliWordExpectations(words, wires)
    for j in range(nwords):
        rj = oracle.expval_pauli_words(psi, [words[j]], [wires[j]], np.array([1.0]))
        assert abs(per[j] - rj) < tol(dtype), (words[j], wires[j], per[j], rj)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [3, 8, 14])
def test_probabilities(native, oracle, dtype, n):
    rng = np.random.default_rng(400 + n)
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    for k in sorted({1, 2, min(n, 5), n - 1, n}):
        for _ in range(2):
            wires = [int(x) for x in rng.choice(n, size=k, replace=False)]
            got = sv.Probability(wires)
            ref = oracle.probs(psi, wires)
            assert np.max(np.abs(got - ref)) < tol(dtype), (wires,)
    got = sv.Probability(sorted(range(n)))
    assert abs(np.sum(got) - 1.0) < tol(dtype) * 10


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [18, 22])
def test_probability_kernel_paths(native, oracle, dtype, n):
    """Every reduction path of lgpu_probs against the oracle: all probed state
    bits >= 10 (per-chunk sums, then one CTA per bin), bits below 8 (a fixed
    bin per thread), bits between 8 and the chunk size (runs of equal bin,
    n = 22), mixed sets, wires in any order, and more than 12 wires (global
    atomics)."""
    rng = np.random.default_rng(900 + n)
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    cases = [[0], [2, 0, 1], list(range(n - 10)), [n - 1], [n - 2, n - 3], [n - 9, n - 10], [n - 12, 1],
             [n - 1, 0, n // 2], list(range(n - 8, n)), list(range(13))]
    for wires in cases:
        got = np.asarray(sv.Probability(wires))
        ref = oracle.probs(psi, wires)
        assert got.shape == ref.shape
        assert np.max(np.abs(got - ref)) < tol(dtype), (wires,)


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [1, 4, 10, 16, 24])
def test_sampling_bit_exact(native, oracle, dtype, n):
    rng = np.random.default_rng(500 + n)
    psi = random_state(n, rng)
    if n >= 4:
        psi[:: 3] = 0  # zero-probability entries must never be drawn
        psi /= np.linalg.norm(psi)
    sv = make_sv(native, dtype, psi)
    seed = 1234 + n
    shots = 3000
    sv.setSeed(seed)
    got = sv.GenerateSampleIndices(shots, True)
    # oracle on the state the device actually holds (c64 rounding included)
    held = sv.GetState().astype(np.complex128)
    ref = oracle.sample_indices(held, seed, shots, float_draws=(dtype == "c64"))
    mism = int(np.sum(got != ref))
    assert mism == 0, "%d of %d samples differ" % (mism, shots)
    assert np.all(np.abs(held[got.astype(np.int64)]) > 0)
    # decoded samples: wire 0 is the most significant bit
    sv.setSeed(seed)
    bits = sv.GenerateSamples(n, shots)
    assert bits.shape == (shots, n)
    assert np.array_equal(bits, oracle.decode_samples(ref, n))


@pytest.mark.gpu
def test_sampling_statistics(native):
    """Histogram of 1e5 shots within 0.05 of |psi|^2 (the reference's own check)."""
    rng = np.random.default_rng(9)
    n = 3
    psi = random_state(n, rng)
    sv = make_sv(native, "c128", psi)
    sv.setSeed(5)
    idx = sv.GenerateSampleIndices(100000, True)
    hist = np.bincount(idx.astype(np.int64), minlength=1 << n) / 1e5
    assert np.max(np.abs(hist - np.abs(psi) ** 2)) < 0.05


@pytest.mark.parametrize("dtype", DTYPES)
def test_sparse_hamiltonian_expval(native, oracle, dtype):
    scipy_sparse = pytest.importorskip("scipy.sparse")
    rng = np.random.default_rng(600)
    n = 6
    psi = random_state(n, rng)
    sv = make_sv(native, dtype, psi)
    h = random_hermitian(1 << n, rng)
    h[np.abs(h) < 0.8] = 0
    h = (h + h.conj().T) / 2
    csr = scipy_sparse.csr_matrix(h)
    itype = np.int64 if dtype == "c128" else np.int32
    got = sv.ExpectationValue(csr.indptr.astype(itype), csr.indices.astype(itype), csr.data.astype(np_dtype(dtype)))
    ref = oracle.expval_sparse(psi, csr.indptr, csr.indices, csr.data)
    assert abs(got - ref) < tol(dtype) * 100


@pytest.mark.parametrize("dtype", DTYPES)
def test_basis_and_state_prep(native, dtype):
    n = 5
    sv = getattr(native, cls_name(dtype))(n)
    sv.setBasisState(13, False)
    st = sv.GetState()
    assert st[13] == 1 and np.count_nonzero(st) == 1
    idx = np.array([1, 5, 30], dtype=np.int64 if dtype == "c128" else np.int32)
    vals = np.array([0.6, 0.8j, 0.0], dtype=np_dtype(dtype))
    sv.setStateVector(idx, vals, False)
    st = sv.GetState()
    assert np.allclose(st[[1, 5, 30]], vals) and np.count_nonzero(st) == 2
    sv.resetGPU()
    st = sv.GetState()
    assert st[0] == 1 and np.count_nonzero(st) == 1


def _obs_native(native, dtype, spec):
    """spec: (is_ham, [(coeff, [(name, wires, matrix)])]) -> native observable."""
    suf = "C128" if dtype == "c128" else "C64"
    is_ham, terms = spec

    def term_obj(factors):
        objs = []
        for name, wires, mat in factors:
            if mat is None:
                objs.append(getattr(native, "NamedObsGPU_" + suf)(name, wires))
            else:
                objs.append(getattr(native, "HermitianObsGPU_" + suf)(np.asarray(mat, np_dtype(dtype)).ravel(), wires))
        return objs[0] if len(objs) == 1 else getattr(native, "TensorProdObsGPU_" + suf)(objs)

    if not is_ham:
        return term_obj(terms[0][1])
    coeffs = np.array([t[0] for t in terms], dtype=np.float64 if dtype == "c128" else np.float32)
    return getattr(native, "HamiltonianGPU_" + suf)(coeffs, [term_obj(t[1]) for t in terms])


ADJ_OPS = ["RX", "RY", "RZ", "PhaseShift", "CRX", "CRY", "CRZ", "ControlledPhaseShift", "IsingXX", "IsingYY",
           "IsingZZ", "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus", "DoubleExcitation",
           "DoubleExcitationMinus", "DoubleExcitationPlus", "MultiRZ"]
NW = {"RX": 1, "RY": 1, "RZ": 1, "PhaseShift": 1, "DoubleExcitation": 4, "DoubleExcitationMinus": 4,
      "DoubleExcitationPlus": 4, "MultiRZ": 3}


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("seed", [0, 1, 2])
def test_adjoint_jacobian_vs_oracle(native, oracle, dtype, seed):
    rng = np.random.default_rng(700 + seed)
    n = 6
    ops = [("Hadamard", [w], [], False) for w in range(n)]
    for name in ADJ_OPS:
        nw = NW.get(name, 2)
        wires = [int(x) for x in rng.choice(n, size=nw, replace=False)]
        ops.append((name, wires, [float(rng.uniform(0, 2 * np.pi))], bool(rng.integers(2))))
        ops.append(("CNOT", [int(x) for x in rng.choice(n, size=2, replace=False)], [], False))
    ops.append(("QubitUnitary", [1, 4], [], False, random_unitary(4, rng)))
    nparam = sum(1 for o in ops if o[2])
    tp = sorted(int(x) for x in rng.choice(nparam, size=min(nparam, 12), replace=False))
    obs_specs = [
        (False, [(1.0, [("PauliZ", [0], None)])]),
        (False, [(1.0, [("PauliX", [1], None), ("PauliY", [3], None)])]),
        (True, [(0.3, [("PauliZ", [2], None)]), (-0.7, [("PauliX", [0], None), ("PauliZ", [5], None)]),
                (0.2, [("PauliY", [4], None)])]),
        (False, [(1.0, [("Hermitian", [2, 5], random_hermitian(4, rng))])]),
        (True, [(0.5, [("Hadamard", [3], None)]), (1.5, [("PauliZ", [1], None)])]),
    ]
    sv = getattr(native, cls_name(dtype))(n)
    apply_ops(sv, ops)
    adj = getattr(native, "AdjointJacobianGPU_" + ("C128" if dtype == "c128" else "C64"))()
    rdt = np.float64 if dtype == "c128" else np.float32
    opsd = adj.create_ops_list([o[0] for o in ops], [np.array(o[2], rdt) for o in ops], [o[1] for o in ops],
                               [o[3] for o in ops],
                               [np.asarray(o[4], np_dtype(dtype)).ravel() if len(o) > 4 else np.zeros(0, np_dtype(dtype))
                                for o in ops])
    obs = [_obs_native(native, dtype, s) for s in obs_specs]
    jac = np.asarray(adj.adjoint_jacobian(sv, obs, opsd, tp))
    final = oracle.run(n, to_oracle_ops(ops))
    oobs = [(s[0], [(c, [(nm, w, m) for nm, w, m in f]) for c, f in s[1]]) for s in obs_specs]
    ref = oracle.adjoint_jacobian(final, to_oracle_ops(ops), oobs, tp)
    assert jac.shape == ref.shape
    assert np.max(np.abs(jac - ref)) < tol(dtype) * 50, np.max(np.abs(jac - ref))


SMALL_ADJ_OPS = ["RX", "RY", "RZ", "PhaseShift", "CRX", "CRY", "CRZ", "ControlledPhaseShift", "IsingXX", "IsingYY",
                 "IsingZZ", "SingleExcitation"]


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [5, 14])
def test_adjoint_sweep_and_step_paths(native, oracle, dtype, n):
    """Operations on at most two wires: n = 5 runs the whole sweep in one
    launch (state in shared memory), n = 14 the per-operation steps; both
    agree with the oracle."""
    rng = np.random.default_rng(900 + n)
    ops = [("Hadamard", [w], [], False) for w in range(n)]
    for rep in range(2):
        for name in SMALL_ADJ_OPS:
            nw = NW.get(name, 2)
            wires = [int(x) for x in rng.choice(n, size=nw, replace=False)]
            ops.append((name, wires, [float(rng.uniform(0, 2 * np.pi))], bool(rng.integers(2))))
            ops.append(("CNOT", [int(x) for x in rng.choice(n, size=2, replace=False)], [], False))
    ops.append(("SWAP", [0, n - 1], [], False))
    nparam = sum(1 for o in ops if o[2])
    tp = sorted(int(x) for x in rng.choice(nparam, size=16, replace=False))
    obs_specs = [
        (False, [(1.0, [("PauliZ", [0], None)])]),
        (False, [(1.0, [("PauliX", [1], None), ("PauliY", [n - 1], None)])]),
        (True, [(0.3, [("PauliZ", [2], None)]), (-0.7, [("PauliX", [0], None), ("PauliZ", [3], None)])]),
    ]
    sv = getattr(native, cls_name(dtype))(n)
    apply_ops(sv, ops)
    adj = getattr(native, "AdjointJacobianGPU_" + ("C128" if dtype == "c128" else "C64"))()
    rdt = np.float64 if dtype == "c128" else np.float32
    opsd = adj.create_ops_list([o[0] for o in ops], [np.array(o[2], rdt) for o in ops], [o[1] for o in ops],
                               [o[3] for o in ops], [np.zeros(0, np_dtype(dtype)) for o in ops])
    obs = [_obs_native(native, dtype, s) for s in obs_specs]
    jac = np.asarray(adj.adjoint_jacobian(sv, obs, opsd, tp))
    final = oracle.run(n, to_oracle_ops(ops))
    oobs = [(s[0], [(c, [(nm, w, m) for nm, w, m in f]) for c, f in s[1]]) for s in obs_specs]
    ref = oracle.adjoint_jacobian(final, to_oracle_ops(ops), oobs, tp)
    assert np.max(np.abs(jac - ref)) < tol(dtype) * 50, np.max(np.abs(jac - ref))


BLOCK_ADJ_OPS = ["RX", "RY", "RZ", "PhaseShift", "CRX", "CRY", "CRZ", "ControlledPhaseShift", "Hadamard", "S", "T",
                 "CNOT", "CZ", "Toffoli", "IsingXX", "SingleExcitation"]


@pytest.mark.parametrize("n,nobs,dtype", [(14, 1, "c128"), (14, 2, "c128"), (14, 3, "c128"), (16, 1, "c128"),
                                          (14, 1, "c64"), (14, 3, "c64")])
def test_adjoint_fused_blocks(native, oracle, n, nobs, dtype):
    """States above the shared-memory sweep run runs of 1-target operations
    (controls allowed) as fused blocks (complex128 in float-float arithmetic,
    complex64 in FP32), up to two observables per pass (three: a pair, then
    the third from the same lambda); non-1-target operations (IsingXX,
    SingleExcitation) end a block and take the per-operation path.  Against
    the oracle adjoint at 50 x the dtype tolerance (1e-10 / 1e-5), with a
    trainable subset."""
    rng = np.random.default_rng(1300 + n + nobs)
    ops = [("Hadamard", [w], [], False) for w in range(n)]
    nw = {"CRX": 2, "CRY": 2, "CRZ": 2, "ControlledPhaseShift": 2, "CNOT": 2, "CZ": 2, "Toffoli": 3, "IsingXX": 2,
          "SingleExcitation": 2}
    for _ in range(60):
        name = BLOCK_ADJ_OPS[int(rng.integers(len(BLOCK_ADJ_OPS)))]
        wires = [int(x) for x in rng.choice(n, size=nw.get(name, 1), replace=False)]
        params = [float(rng.uniform(0, 2 * np.pi))] if name not in ("Hadamard", "S", "T", "CNOT", "CZ", "Toffoli") else []
        ops.append((name, wires, params, bool(rng.integers(2)) and bool(params)))
    nparam = sum(1 for o in ops if o[2])
    tp = sorted(int(x) for x in rng.choice(nparam, size=min(24, nparam), replace=False))
    obs_specs = [(True, [(0.6, [("PauliZ", [1], None)]), (-0.4, [("PauliX", [0], None), ("PauliY", [n - 1], None)])]),
                 (False, [(1.0, [("PauliY", [3], None)])]),
                 (False, [(1.0, [("PauliX", [n - 2], None), ("PauliZ", [5], None)])])][:nobs]
    suf = "C128" if dtype == "c128" else "C64"
    rdt = np.float64 if dtype == "c128" else np.float32
    sv = getattr(native, cls_name(dtype))(n)
    apply_ops(sv, ops)
    adj = getattr(native, "AdjointJacobianGPU_" + suf)()
    opsd = adj.create_ops_list([o[0] for o in ops], [np.array(o[2], rdt) for o in ops], [o[1] for o in ops],
                               [o[3] for o in ops], [np.zeros(0, np_dtype(dtype)) for o in ops])
    obs = [_obs_native(native, dtype, s) for s in obs_specs]
    jac = np.asarray(adj.adjoint_jacobian(sv, obs, opsd, tp))
    final = oracle.run(n, to_oracle_ops(ops))
    oobs = [(s[0], [(c, [(nm, w, m) for nm, w, m in f]) for c, f in s[1]]) for s in obs_specs]
    ref = oracle.adjoint_jacobian(final, to_oracle_ops(ops), oobs, tp)
    assert np.max(np.abs(jac - ref)) < tol(dtype) * 50, np.max(np.abs(jac - ref))
    assert np.max(np.abs(ref)) > 1e-3  # the circuit has gradients to compare


@pytest.mark.parametrize("n,nobs,dtype", [(14, 1, "c128"), (14, 2, "c128"), (15, 3, "c128"), (14, 1, "c64"),
                                          (15, 3, "c64")])
def test_adjoint_phase_groups(native, oracle, n, nobs, dtype):
    """Fused adjoint blocks (complex128 and complex64) take runs of uncontrolled diagonal
    steps (RZ, PhaseShift, trainable or not, adjoint or not) on up to 4 tile
    positions as phase groups: one overlap product per amplitude for all of
    them, then one phase table.  Layers of RY / RZ / PhaseShift runs with CZ
    and CNOT between them, a trainable subset, 1 to 3 observables: against
    the oracle adjoint at 50 x the dtype tolerance (1e-10 / 1e-5)."""
    rng = np.random.default_rng(4100 + n + nobs)
    ops = [("Hadamard", [w], [], False) for w in range(n)]
    for layer in range(4):
        for w in range(n):
            ops.append(("RY", [w], [float(rng.uniform(0, 2 * np.pi))], bool(rng.integers(2))))
        for w in rng.permutation(n):  # diagonal runs, several gates on one wire at times
            name = ("RZ", "PhaseShift")[int(rng.integers(2))]
            ops.append((name, [int(w)], [float(rng.uniform(0, 2 * np.pi))], bool(rng.integers(2))))
            if rng.integers(4) == 0:
                ops.append(("RZ", [int(w)], [float(rng.uniform(0, 2 * np.pi))], False))
        for w in range(0, n - 1, 2):
            ops.append((("CZ", "CNOT")[layer % 2], [w, w + 1], [], False))
    nparam = sum(1 for o in ops if o[2])
    tp = sorted(int(x) for x in rng.choice(nparam, size=nparam * 2 // 3, replace=False))
    obs_specs = [(True, [(0.6, [("PauliZ", [1], None)]), (-0.4, [("PauliX", [0], None), ("PauliY", [n - 1], None)])]),
                 (False, [(1.0, [("PauliY", [3], None)])]),
                 (False, [(1.0, [("PauliX", [n - 2], None), ("PauliZ", [5], None)])])][:nobs]
    suf = "C128" if dtype == "c128" else "C64"
    rdt = np.float64 if dtype == "c128" else np.float32
    sv = getattr(native, cls_name(dtype))(n)
    apply_ops(sv, ops)
    adj = getattr(native, "AdjointJacobianGPU_" + suf)()
    opsd = adj.create_ops_list([o[0] for o in ops], [np.array(o[2], rdt) for o in ops], [o[1] for o in ops],
                               [o[3] for o in ops], [np.zeros(0, np_dtype(dtype)) for o in ops])
    obs = [_obs_native(native, dtype, s) for s in obs_specs]
    jac = np.asarray(adj.adjoint_jacobian(sv, obs, opsd, tp))
    final = oracle.run(n, to_oracle_ops(ops))
    oobs = [(s[0], [(c, [(nm, w, m) for nm, w, m in f]) for c, f in s[1]]) for s in obs_specs]
    ref = oracle.adjoint_jacobian(final, to_oracle_ops(ops), oobs, tp)
    assert np.max(np.abs(jac - ref)) < tol(dtype) * 50, np.max(np.abs(jac - ref))
    assert np.max(np.abs(ref)) > 1e-3


@pytest.mark.parametrize("dtype", DTYPES)
def test_adjoint_rejects_multiparam(native, dtype):
    suf = "C128" if dtype == "c128" else "C64"
    rdt = np.float64 if dtype == "c128" else np.float32
    sv = getattr(native, cls_name(dtype))(2)
    adj = getattr(native, "AdjointJacobianGPU_" + suf)()
    opsd = adj.create_ops_list(["Rot"], [np.array([0.1, 0.2, 0.3], rdt)], [[0]], [False], [np.zeros(0, np_dtype(dtype))])
    with pytest.raises(native.PLException, match="not supported using the adjoint"):
        adj.adjoint_jacobian(sv, [getattr(native, "NamedObsGPU_" + suf)("PauliZ", [0])], opsd, [0])


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("name,nw,npar", [g for g in GATES if g[1] <= 2])
def test_f64_modes(native, oracle, mode, name, nw, npar):
    """complex128 gates agree with the oracle with native FP64 and with the
    integer-pipe multiplies."""
    old = native.get_f64_mode()
    native.set_f64_mode(mode)
    try:
        rng = np.random.default_rng(zlib.crc32(("mode-%s-%d" % (name, mode)).encode()))
        n = 8
        for _ in range(3):
            wires = [int(x) for x in rng.choice(n, size=nw, replace=False)]
            params = [float(x) for x in rng.uniform(0, 2 * np.pi, npar)]
            for adj in (False, True):
                _check(native, oracle, "c128", n, [(name, wires, params, adj)], rng)
    finally:
        native.set_f64_mode(old)


def test_f64_mode_bits_close(native):
    """The two complex128 modes differ by at most a few ulp after many gates."""
    from pennylane_lightning_gpu_gb300 import workloads

    rng = np.random.default_rng(5)
    n = 12
    ops = workloads.layered_ansatz(n, 6, rng) + [("Hadamard", [w], [], False) for w in range(n)]
    psi = random_state(n, rng)
    out = []
    old = native.get_f64_mode()
    try:
        for mode in (0, 1):
            native.set_f64_mode(mode)
            sv = make_sv(native, "c128", psi)
            sv.setFusion(False)
            apply_ops(sv, ops)
            out.append(sv.GetState())
    finally:
        native.set_f64_mode(old)
    assert np.max(np.abs(out[0] - out[1])) < 1e-13


@pytest.mark.parametrize("dtype", DTYPES)
@pytest.mark.parametrize("n", [14, 16])
def test_bulk_stream_kernel_all_targets(native, oracle, dtype, n):
    """The bulk-copy pipelined 1-target kernel (split and interleaved tiles,
    every body) against the oracle and the grid-stride kernel."""
    rng = np.random.default_rng(900 + n)
    psi = random_state(n, rng)
    gates = [("Hadamard", []), ("RX", [0.3]), ("RY", [1.1]), ("RZ", [2.2]), ("PauliX", []), ("PauliY", []),
             ("Rot", [0.2, 0.5, 0.9])]
    ops = []
    for w in range(n):
        g, par = gates[w % len(gates)]
        ops.append((g, [w], par, bool(w % 2)))
    old = native.get_stream_mode()
    outs = []
    try:
        for mode in (1, 0):
            native.set_stream_mode(mode)
            sv = make_sv(native, dtype, psi)
            apply_ops(sv, ops)
            outs.append(sv.GetState())
    finally:
        native.set_stream_mode(old)
    ref = oracle.apply_ops(psi, to_oracle_ops(ops))
    assert np.max(np.abs(outs[0] - ref)) < tol(dtype)
    assert np.max(np.abs(outs[1] - ref)) < tol(dtype)

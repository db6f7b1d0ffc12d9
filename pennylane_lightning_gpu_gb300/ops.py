"""A minimal operation / observable / tape model with PennyLane's names.

PennyLane is not a dependency of this engine, so the Python device works on
these small classes instead of ``qml.operation`` objects.  They carry what
the reference device reads from PennyLane objects: ``name``, ``wires``,
``parameters``, ``matrix()``, ``diagonalizing_gates()`` for observables,
and, for tapes, ``operations``, ``measurements``, ``observables`` and
``trainable_params``.  Matrices follow PennyLane's convention (row-major,
first wire most significant).
"""
from functools import reduce

import numpy as np

_SQ2 = 1.0 / np.sqrt(2.0)


def _rx(t):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return np.array([[c, -1j * s], [-1j * s, c]])


def _ry(t):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return np.array([[c, -s], [s, c]], dtype=complex)


def _rz(t):
    return np.diag([np.exp(-0.5j * t), np.exp(0.5j * t)])


def _ctrl(u, nctrl=1):
    d = u.shape[0]
    m = np.eye(d << nctrl, dtype=complex)
    m[-d:, -d:] = u
    return m


def _pauli_word_matrix(word):
    mats = {"I": np.eye(2), "X": np.array([[0, 1], [1, 0]]), "Y": np.array([[0, -1j], [1j, 0]]),
            "Z": np.diag([1, -1])}
    return reduce(np.kron, [mats[c] for c in word]).astype(complex)


def _rot(phi, theta, omega):
    return _rz(omega) @ _ry(theta) @ _rz(phi)


def _single_exc(t, outer=1.0):
    c, s = np.cos(t / 2), np.sin(t / 2)
    return np.array([[outer, 0, 0, 0], [0, c, -s, 0], [0, s, c, 0], [0, 0, 0, outer]], dtype=complex)


def _double_exc(t, outer=1.0):
    c, s = np.cos(t / 2), np.sin(t / 2)
    m = np.eye(16, dtype=complex) * outer
    m[3, 3], m[3, 12], m[12, 3], m[12, 12] = c, -s, s, c
    return m


def _multirz(t, k):
    z = np.array([1.0])
    for _ in range(k):
        z = np.kron(z, np.array([1.0, -1.0]))
    return np.diag(np.exp(-0.5j * t * z))


def _qft(k):
    """Quantum Fourier transform on k wires: (1/sqrt(N)) w^(r c), w = exp(2 pi i / N)."""
    d = 1 << k
    rc = np.outer(np.arange(d), np.arange(d)) % d
    return np.exp(2j * np.pi * rc / d) / np.sqrt(d)


def _grover(k):
    """Grover diffusion operator on k wires: 2 |s><s| - I, |s> the uniform superposition."""
    d = 1 << k
    return np.full((d, d), 2.0 / d, dtype=complex) - np.eye(d)


_MATRICES = {
    "Identity": lambda p, k: np.eye(2, dtype=complex),
    "PauliX": lambda p, k: np.array([[0, 1], [1, 0]], dtype=complex),
    "PauliY": lambda p, k: np.array([[0, -1j], [1j, 0]]),
    "PauliZ": lambda p, k: np.diag([1.0, -1.0]).astype(complex),
    "Hadamard": lambda p, k: np.array([[_SQ2, _SQ2], [_SQ2, -_SQ2]], dtype=complex),
    "S": lambda p, k: np.diag([1, 1j]),
    "T": lambda p, k: np.diag([1, np.exp(0.25j * np.pi)]),
    "SX": lambda p, k: 0.5 * np.array([[1 + 1j, 1 - 1j], [1 - 1j, 1 + 1j]]),
    "RX": lambda p, k: _rx(p[0]),
    "RY": lambda p, k: _ry(p[0]),
    "RZ": lambda p, k: _rz(p[0]),
    "PhaseShift": lambda p, k: np.diag([1, np.exp(1j * p[0])]),
    "Rot": lambda p, k: _rot(*p),
    "CNOT": lambda p, k: _ctrl(np.array([[0, 1], [1, 0]], dtype=complex)),
    "CY": lambda p, k: _ctrl(np.array([[0, -1j], [1j, 0]])),
    "CZ": lambda p, k: _ctrl(np.diag([1.0, -1.0]).astype(complex)),
    "SWAP": lambda p, k: np.eye(4, dtype=complex)[[0, 2, 1, 3]],
    "CSWAP": lambda p, k: _ctrl(np.eye(4, dtype=complex)[[0, 2, 1, 3]]),
    "Toffoli": lambda p, k: _ctrl(np.array([[0, 1], [1, 0]], dtype=complex), 2),
    "CRX": lambda p, k: _ctrl(_rx(p[0])),
    "CRY": lambda p, k: _ctrl(_ry(p[0])),
    "CRZ": lambda p, k: _ctrl(_rz(p[0])),
    "CRot": lambda p, k: _ctrl(_rot(*p)),
    "ControlledPhaseShift": lambda p, k: _ctrl(np.diag([1, np.exp(1j * p[0])])),
    "IsingXX": lambda p, k: np.cos(p[0] / 2) * np.eye(4) - 1j * np.sin(p[0] / 2) * _pauli_word_matrix("XX"),
    "IsingYY": lambda p, k: np.cos(p[0] / 2) * np.eye(4) - 1j * np.sin(p[0] / 2) * _pauli_word_matrix("YY"),
    "IsingZZ": lambda p, k: _multirz(p[0], 2),
    "MultiRZ": lambda p, k: _multirz(p[0], k),
    "SingleExcitation": lambda p, k: _single_exc(p[0]),
    "SingleExcitationMinus": lambda p, k: _single_exc(p[0], np.exp(-0.5j * p[0])),
    "SingleExcitationPlus": lambda p, k: _single_exc(p[0], np.exp(0.5j * p[0])),
    "DoubleExcitation": lambda p, k: _double_exc(p[0]),
    "DoubleExcitationMinus": lambda p, k: _double_exc(p[0], np.exp(-0.5j * p[0])),
    "DoubleExcitationPlus": lambda p, k: _double_exc(p[0], np.exp(0.5j * p[0])),
    "QFT": lambda p, k: _qft(k),
    "GroverOperator": lambda p, k: _grover(k),
}

_NUM_PARAMS = {"RX": 1, "RY": 1, "RZ": 1, "PhaseShift": 1, "Rot": 3, "CRX": 1, "CRY": 1, "CRZ": 1, "CRot": 3,
               "ControlledPhaseShift": 1, "IsingXX": 1, "IsingYY": 1, "IsingZZ": 1, "MultiRZ": 1,
               "SingleExcitation": 1, "SingleExcitationMinus": 1, "SingleExcitationPlus": 1, "DoubleExcitation": 1,
               "DoubleExcitationMinus": 1, "DoubleExcitationPlus": 1}


class Operation:
    """A gate: name, wires, parameters (and an explicit matrix for unnamed gates)."""

    is_observable = False

    def __init__(self, name, wires, params=(), matrix=None):
        self.name = name
        self.wires = [wires] if isinstance(wires, (int, np.integer)) else list(wires)
        self.parameters = [float(p) for p in np.atleast_1d(params)] if len(np.atleast_1d(params)) else []
        self._matrix = None if matrix is None else np.asarray(matrix, dtype=complex)

    @property
    def num_params(self):
        return len(self.parameters)

    def matrix(self):
        if self._matrix is not None:
            return self._matrix
        if self.name not in _MATRICES:
            raise ValueError("no matrix for %s" % self.name)
        return np.asarray(_MATRICES[self.name](self.parameters, len(self.wires)), dtype=complex)

    def adjoint(self):
        return Adjoint(self)

    def __repr__(self):
        return "%s(%s, wires=%s)" % (self.name, self.parameters, self.wires)


class Adjoint(Operation):
    """Adjoint of an operation (``name`` stays the base name, as the device
    reads ``o.base.name``)."""

    def __init__(self, base):
        super().__init__(base.name, base.wires, base.parameters, base._matrix)
        self.base = base

    def matrix(self):
        return self.base.matrix().conj().T


def op(name, wires, *params, matrix=None):
    return Operation(name, wires, params, matrix)


def QubitUnitary(U, wires):
    return Operation("QubitUnitary", wires, (), U)


def QFT(wires):
    return Operation("QFT", wires)


def GroverOperator(wires):
    return Operation("GroverOperator", wires)


class StatePrep(Operation):
    def __init__(self, state, wires):
        super().__init__("StatePrep", wires)
        self.state = np.asarray(state, dtype=complex)


class BasisState(Operation):
    def __init__(self, bits, wires):
        super().__init__("BasisState", wires)
        self.bits = [int(b) for b in bits]


# ---- observables -----------------------------------------------------------
class Observable:
    is_observable = True

    def __init__(self, name, wires, params=(), matrix=None):
        self.name = name
        self.wires = [wires] if isinstance(wires, (int, np.integer)) else list(wires)
        self.parameters = list(params)
        self._matrix = None if matrix is None else np.asarray(matrix, dtype=complex)

    def matrix(self):
        if self._matrix is not None:
            return self._matrix
        return np.asarray(_MATRICES[self.name](self.parameters, len(self.wires)), dtype=complex)

    def eigvals(self):
        return np.linalg.eigvalsh(self.matrix())

    def diagonalizing_gates(self):
        if self.name == "PauliX":
            return [op("Hadamard", self.wires)]
        if self.name == "PauliY":
            return [op("PauliZ", self.wires), op("S", self.wires), op("Hadamard", self.wires)]
        if self.name == "Hadamard":
            return [op("RY", self.wires, -np.pi / 4)]
        if self.name in ("PauliZ", "Identity"):
            return []
        w, v = np.linalg.eigh(self.matrix())
        return [QubitUnitary(v.conj().T, self.wires)]

    def __matmul__(self, other):
        return Tensor(self, other)

    def __repr__(self):
        return "%s(wires=%s)" % (self.name, self.wires)


def PauliX(w):
    return Observable("PauliX", w)


def PauliY(w):
    return Observable("PauliY", w)


def PauliZ(w):
    return Observable("PauliZ", w)


def Hadamard(w):
    return Observable("Hadamard", w)


def Identity(w):
    return Observable("Identity", w)


def Hermitian(matrix, wires):
    return Observable("Hermitian", wires, (), matrix)


class Projector(Observable):
    def __init__(self, basis_state, wires):
        super().__init__("Projector", wires)
        self.basis_state = [int(b) for b in basis_state]

    def matrix(self):
        d = 1 << len(self.wires)
        m = np.zeros((d, d), dtype=complex)
        idx = int("".join(str(b) for b in self.basis_state), 2)
        m[idx, idx] = 1
        return m


class Tensor(Observable):
    def __init__(self, *obs):
        flat = []
        for o in obs:
            flat.extend(o.obs if isinstance(o, Tensor) else [o])
        self.obs = flat
        wires = [w for o in flat for w in o.wires]
        if len(set(wires)) != len(wires):
            raise ValueError("All wires in observables must be disjoint.")
        super().__init__([o.name for o in flat], wires)

    @property
    def non_identity_obs(self):
        return [o for o in self.obs if o.name != "Identity"]

    def matrix(self):
        return reduce(np.kron, [o.matrix() for o in self.obs])

    def diagonalizing_gates(self):
        return [g for o in self.obs for g in o.diagonalizing_gates()]

    def __matmul__(self, other):
        return Tensor(self, other)


class Hamiltonian(Observable):
    def __init__(self, coeffs, observables):
        self.coeffs = np.asarray(coeffs, dtype=float)
        self.ops = list(observables)
        if len(self.coeffs) != len(self.ops):
            raise ValueError("number of coefficients and observables differ")
        # PennyLane's order: wires in order of first appearance (any hashable labels)
        wires = list(dict.fromkeys(w for o in self.ops for w in o.wires))
        super().__init__("Hamiltonian", wires)

    def matrix(self, wire_order=None):
        wires = self.wires if wire_order is None else list(wire_order)
        n = len(wires)
        total = np.zeros((1 << n, 1 << n), dtype=complex)
        for c, o in zip(self.coeffs, self.ops):
            total += c * embed(o.matrix(), o.wires, wires)
        return total


class SparseHamiltonian(Observable):
    def __init__(self, csr, wires):
        super().__init__("SparseHamiltonian", wires)
        self.csr = csr

    def sparse_matrix(self):
        return self.csr


def embed(mat, op_wires, all_wires):
    """Matrix of `mat` (on op_wires) embedded on all_wires (first = MSB)."""
    n = len(all_wires)
    k = len(op_wires)
    pos = [all_wires.index(w) for w in op_wires]
    rest = [i for i in range(n) if i not in pos]
    full = np.zeros((1 << n, 1 << n), dtype=complex)
    for r in range(1 << n):
        rb = [(r >> (n - 1 - i)) & 1 for i in range(n)]
        rsub = int("".join(str(rb[p]) for p in pos), 2) if k else 0
        for cs in range(1 << k):
            cb = list(rb)
            for j, p in enumerate(pos):
                cb[p] = (cs >> (k - 1 - j)) & 1
            c = int("".join(str(b) for b in cb), 2)
            full[r, c] = mat[rsub, cs]
    return full


# ---- measurements and tapes -------------------------------------------------
class MeasurementProcess:
    def __init__(self, return_type, obs=None, wires=None):
        self.return_type = return_type
        self.obs = obs
        self.wires = list(wires) if wires is not None else (obs.wires if obs is not None else None)


def expval(obs):
    return MeasurementProcess("expval", obs)


def var(obs):
    return MeasurementProcess("var", obs)


def probs(wires=None):
    return MeasurementProcess("probs", None, wires)


def sample(obs=None, wires=None):
    return MeasurementProcess("sample", obs, wires)


def state():
    return MeasurementProcess("state")


class QuantumTape:
    def __init__(self, operations, measurements, trainable_params=None):
        self.operations = list(operations)
        self.measurements = list(measurements)
        if trainable_params is None:
            trainable_params = list(range(sum(len(o.parameters) for o in self.operations
                                              if not isinstance(o, (StatePrep, BasisState)))))
        self.trainable_params = list(trainable_params)

    @property
    def observables(self):
        return [m.obs for m in self.measurements]

    def get_parameters(self):
        return [p for o in self.operations for p in o.parameters]

    def get_operation(self, idx):
        """Operation owning the idx-th trainable parameter, and its local index."""
        t = self.trainable_params[idx]
        owners = self._param_owners()
        if not 0 <= t < len(owners):
            raise IndexError(idx)
        o, j = owners[t]
        return o, t, j

    def _param_owners(self):
        """(operation, local index) of every parameter, built once per tape."""
        owners = getattr(self, "_owners", None)
        if owners is None:
            owners = [(o, j) for o in self.operations if not isinstance(o, (StatePrep, BasisState))
                      for j in range(len(o.parameters))]
            self._owners = owners
        return owners

    def copy(self):
        return QuantumTape(self.operations, self.measurements, self.trainable_params)

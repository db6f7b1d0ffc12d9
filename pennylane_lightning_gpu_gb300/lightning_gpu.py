"""LightningGPU: the Python device of the GB300 engine.

Mirrors the hot-path methods of the reference device
(pennylane_lightning_gpu/lightning_gpu.py:205-973): ``apply`` / ``apply_cq``,
``expval``, ``var``, ``probability``, ``generate_samples``, ``sample``,
``adjoint_jacobian`` and ``vjp``, plus ``execute`` for whole tapes.  It works
on the small op/observable/tape classes of ``ops.py`` (PennyLane itself is not
a dependency) and drives the native ``LightningGPU_C64/C128`` state vector.

Deliberate differences from the reference (each noted where it happens):
  * no CPU fall-back: without the CUDA extension or a GPU the device raises;
  * ``mpi=True`` raises (everything runs on one GPU);
  * ``apply_cq`` inverts only the ``Adjoint`` operations themselves (the
    reference's flag stays set for every later operation);
  * the complex64 adjoint path no longer reads an unassigned ``ket``;
  * multi-operation ``apply`` uses the shared-memory gate-fusion path;
  * Hamiltonian expectation values always use the Pauli-word kernels (the
    reference builds a dense matrix on the host below 14 wires).
"""
import warnings

import numpy as np

from . import ops as Q
from ._native import native
from ._serialize import _expanded_param_positions, _serialize_observables, _serialize_ops

_NAME_MAP = {"PauliX": "X", "PauliY": "Y", "PauliZ": "Z", "Identity": "I"}


class DeviceError(Exception):
    pass


class QuantumFunctionError(Exception):
    pass


class LightningGPU:
    name = "GB300 statevector engine with the LightningGPU interface"
    short_name = "lightning.gpu"

    operations = {"Identity", "BasisState", "QubitStateVector", "StatePrep", "QubitUnitary", "PauliX", "PauliY",
                  "PauliZ", "Hadamard", "S", "T", "SX", "CNOT", "SWAP", "CSWAP", "Toffoli", "CY", "CZ", "PhaseShift",
                  "ControlledPhaseShift", "RX", "RY", "RZ", "Rot", "CRX", "CRY", "CRZ", "CRot", "IsingXX", "IsingYY",
                  "IsingZZ", "MultiRZ", "SingleExcitation", "SingleExcitationMinus", "SingleExcitationPlus",
                  "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus", "QFT", "GroverOperator"}
    # dense matrix operations and the widest register the device applies them
    # to directly (reference stopping_condition, lightning_gpu.py:504-511);
    # wider ones must be decomposed before they reach the device
    matrix_operations = {"QFT": 9, "GroverOperator": 12}
    observables = {"PauliX", "PauliY", "PauliZ", "Hadamard", "Identity", "Hermitian", "Projector", "Hamiltonian",
                   "SparseHamiltonian"}

    def __init__(self, wires, *, c_dtype=np.complex128, shots=None, batch_obs=False, mpi=False, sync=False,
                 seed=None, fusion=True, adjoint_hermitian=False):
        if mpi:
            raise DeviceError("mpi=True is not supported: the GB300 engine runs one state on one GPU")
        if c_dtype not in (np.complex64, np.complex128):
            raise TypeError("Unsupported complex Type: %s" % c_dtype)
        self.wires = list(range(wires)) if isinstance(wires, int) else list(wires)
        self.num_wires = len(self.wires)
        self.wire_map = {w: i for i, w in enumerate(self.wires)}
        self.C_DTYPE = c_dtype
        self.R_DTYPE = np.float32 if c_dtype == np.complex64 else np.float64
        self.use_csingle = c_dtype == np.complex64
        self.shots = shots
        self._batch_obs = batch_obs
        self._sync = sync
        self._mod = native()
        self._gpu_state = getattr(self._mod, "LightningGPU_C64" if self.use_csingle else "LightningGPU_C128")(
            self.num_wires)
        self._gpu_state.setFusion(bool(fusion))
        if seed is not None:
            self._gpu_state.setSeed(int(seed))
        self._samples = None
        # The reference refuses Hermitian observables in adjoint differentiation
        # (lightning_gpu.py:606-618); the engine supports them when asked.
        self._adjoint_hermitian = bool(adjoint_hermitian)

    # ------------------------------------------------------------------ state
    def reset(self):
        self._gpu_state.resetGPU()
        self._samples = None

    def map_wires(self, wires):
        return [self.wire_map[w] for w in wires]

    @property
    def state(self):
        return self._gpu_state.GetState()

    def syncH2D(self, state_vector, use_async=False):
        self._gpu_state.HostToDevice(np.ascontiguousarray(np.ravel(state_vector), self.C_DTYPE), use_async)

    def syncD2H(self, state_vector, use_async=False):
        self._gpu_state.DeviceToHost(state_vector.ravel(order="C"), use_async)

    def _apply_state_vector_GPU(self, state, device_wires):
        """StatePrep: full-wire states go through HostToDevice, partial-wire
        states through the device scatter (reference lightning_gpu.py:392-447)."""
        device_wires = self.map_wires(device_wires)
        dim = 2 ** len(device_wires)
        state = np.asarray(state, dtype=self.C_DTYPE)
        if state.shape != (dim,):
            raise ValueError("State vector must have shape (2**wires,) or (batch_size, 2**wires).")
        if not np.allclose(np.linalg.norm(state), 1.0, atol=1e-6):
            raise ValueError("Sum of amplitudes-squared does not equal one.")
        if len(device_wires) == self.num_wires and sorted(device_wires) == device_wires:
            self.syncH2D(state)
            return
        n = self.num_wires
        idx = np.zeros(dim, dtype=np.int64)
        for k in range(dim):
            full = 0
            for j, w in enumerate(device_wires):
                if (k >> (len(device_wires) - 1 - j)) & 1:
                    full |= 1 << (n - 1 - w)
            idx[k] = full
        itype = np.int32 if self.use_csingle else np.int64
        self._gpu_state.setStateVector(idx.astype(itype), state, False)

    def _apply_basis_state_GPU(self, state, wires):
        device_wires = self.map_wires(wires)
        state = list(state)
        if not set(state).issubset({0, 1}):
            raise ValueError("BasisState parameter must consist of 0 or 1 integers.")
        if len(state) != len(device_wires):
            raise ValueError("BasisState parameter and wires must be of equal length.")
        num = int(sum(b << (self.num_wires - 1 - w) for b, w in zip(state, device_wires)))
        self._gpu_state.setBasisState(num, False)

    # ------------------------------------------------------------------ apply
    def apply_cq(self, operations, **kwargs):
        for o in operations:
            if o.name == "Identity":
                continue
            invert = isinstance(o, Q.Adjoint)
            method = getattr(self._gpu_state, o.name, None)
            wires = self.map_wires(o.wires)
            if method is None or o.name == "QubitUnitary":
                mat = o.matrix()
                if len(mat) == 0:
                    raise Exception("Unsupported operation")
                self._gpu_state.apply(o.name, wires, False, [], np.asarray(mat, self.C_DTYPE).ravel(order="C"))
            else:
                method(wires, invert, o.parameters)

    def supports_operation(self, op):
        """True when the device applies `op` itself (name known; QFT below 10
        wires, GroverOperator below 13, as the reference's stopping condition)."""
        name = op if isinstance(op, str) else op.name
        if name not in self.operations:
            return False
        limit = self.matrix_operations.get(name)
        return limit is None or isinstance(op, str) or len(op.wires) <= limit

    def apply(self, operations, **kwargs):
        for o in operations:
            limit = self.matrix_operations.get(o.name)
            if limit is not None and len(o.wires) > limit:
                raise DeviceError("%s on %d wires is not applied by the device (at most %d wires): decompose it "
                                  "first" % (o.name, len(o.wires), limit))
        if operations:
            if isinstance(operations[0], Q.StatePrep):
                self._apply_state_vector_GPU(operations[0].state, operations[0].wires)
                operations = operations[1:]
            elif isinstance(operations[0], Q.BasisState):
                self._apply_basis_state_GPU(operations[0].bits, operations[0].wires)
                operations = operations[1:]
        for o in operations:
            if isinstance(o, (Q.StatePrep, Q.BasisState)):
                raise DeviceError("Operation %s cannot be used after other Operations have already been applied "
                                  "on a %s device." % (o.name, self.short_name))
        named = all(getattr(self._gpu_state, o.name, None) is not None and o.name != "QubitUnitary"
                    for o in operations)
        if named and len(operations) > 1:
            # one call: the engine lowers, fuses and applies the whole list
            self._gpu_state.apply([o.name for o in operations], [self.map_wires(o.wires) for o in operations],
                                  [isinstance(o, Q.Adjoint) for o in operations],
                                  [list(o.parameters) for o in operations])
        else:
            self.apply_cq(operations)

    # ------------------------------------------------------------ statistics
    def expval(self, observable, shot_range=None, bin_size=None):
        if observable.name == "Projector":
            p = self.probability(observable.wires)
            return float(p[int("".join(str(b) for b in observable.basis_state), 2)])
        if self.shots is not None:
            samples = self.sample(observable)
            return np.squeeze(np.mean(samples, axis=0))
        if observable.name == "SparseHamiltonian":
            csr = observable.sparse_matrix().tocsr()
            itype = np.int32 if self.use_csingle else np.int64
            return self._gpu_state.ExpectationValue(csr.indptr.astype(itype), csr.indices.astype(itype),
                                                    csr.data.astype(self.C_DTYPE))
        if observable.name == "Hamiltonian":
            words, word_wires, coeffs = self._pauli_words(observable)
            if words is not None:
                return self._gpu_state.ExpectationValue(words, word_wires, np.asarray(coeffs, self.C_DTYPE))
            return self._gpu_state.ExpectationValue(self.map_wires(observable.wires),
                                                    observable.matrix().astype(self.C_DTYPE).ravel(order="C"))
        if observable.name == "Hermitian":
            return self._gpu_state.ExpectationValue(self.map_wires(observable.wires),
                                                    observable.matrix().astype(self.C_DTYPE).ravel(order="C"))
        names = observable.name if isinstance(observable.name, list) else None
        if names is not None:
            return self._gpu_state.ExpectationValue(names, self.map_wires(observable.wires), [[] for _ in names],
                                                    observable.matrix().astype(self.C_DTYPE).ravel(order="C"))
        return self._gpu_state.ExpectationValue(observable.name, self.map_wires(observable.wires), [],
                                                observable.matrix().astype(self.C_DTYPE).ravel(order="C"))

    def _pauli_words(self, ham):
        words, word_wires = [], []
        for term in ham.ops:
            parts = term.obs if isinstance(term, Q.Tensor) else [term]
            w = ""
            for p in parts:
                if p.name not in _NAME_MAP:
                    return None, None, None
                w += _NAME_MAP[p.name]
            words.append(w)
            word_wires.append(self.map_wires([x for p in parts for x in p.wires]))
        return words, word_wires, list(ham.coeffs)

    def var(self, observable, shot_range=None, bin_size=None):
        if self.shots is not None:
            samples = self.sample(observable)
            return np.squeeze(np.var(samples, axis=0))
        mat = observable.matrix()
        sqr = mat.conj().T @ mat
        wires = self.map_wires(observable.wires)
        mean = self._gpu_state.ExpectationValue(wires, mat.astype(self.C_DTYPE).ravel(order="C"))
        squared_mean = self._gpu_state.ExpectationValue(wires, sqr.astype(self.C_DTYPE).ravel(order="C"))
        return squared_mean - mean ** 2

    def probability(self, wires=None, shot_range=None, bin_size=None):
        if self.shots is not None:
            return self.estimate_probability(wires)
        wires = self.wires if wires is None else list(wires)
        device_wires = self.map_wires(wires)
        if len(device_wires) > 1 and not np.all(np.array(device_wires)[:-1] <= np.array(device_wires)[1:]):
            raise RuntimeError("Lightning does not currently support out-of-order indices for probabilities")
        local_prob = self._gpu_state.Probability(device_wires)
        if len(local_prob) > 0:
            k = len(local_prob).bit_length() - 1
            return local_prob.reshape([2] * k).transpose().reshape(-1)
        return local_prob

    def generate_samples(self):
        return self._gpu_state.GenerateSamples(self.num_wires, self.shots).astype(int)

    def estimate_probability(self, wires=None):
        samples = self.generate_samples() if self._samples is None else self._samples
        wires = self.wires if wires is None else list(wires)
        cols = self.map_wires(wires)
        idx = np.zeros(samples.shape[0], dtype=np.int64)
        for c in cols:
            idx = (idx << 1) | samples[:, c]
        return np.bincount(idx, minlength=1 << len(cols)) / samples.shape[0]

    def sample(self, observable, shot_range=None, bin_size=None, counts=False):
        if observable.name != "PauliZ":
            self.apply_cq(observable.diagonalizing_gates())
            self._samples = self.generate_samples()
        elif self._samples is None:
            self._samples = self.generate_samples()
        cols = self.map_wires(observable.wires)
        bits = self._samples[:, cols]
        if observable.name in ("PauliX", "PauliY", "PauliZ", "Hadamard") or (
                isinstance(observable.name, list) and all(n in _NAME_MAP or n == "Hadamard" for n in observable.name)):
            return np.prod(1 - 2 * bits, axis=1)
        eig = np.linalg.eigvalsh(observable.matrix())
        idx = np.zeros(bits.shape[0], dtype=np.int64)
        for c in range(bits.shape[1]):
            idx = (idx << 1) | bits[:, c]
        return eig[idx]

    # -------------------------------------------------------------- execute
    def execute(self, tape):
        self.reset()
        self.apply(tape.operations)
        self._samples = None
        out = []
        for m in tape.measurements:
            if m.return_type == "expval":
                out.append(self.expval(m.obs))
            elif m.return_type == "var":
                out.append(self.var(m.obs))
            elif m.return_type == "probs":
                out.append(self.probability(m.wires))
            elif m.return_type == "sample":
                out.append(self.sample(m.obs) if m.obs is not None else self.generate_samples())
            elif m.return_type == "state":
                out.append(self.state)
        return out

    def batch_execute(self, tapes):
        return [self.execute(t) for t in tapes]

    # ---------------------------------------------------------------- adjoint
    @staticmethod
    def _check_adjdiff_supported_measurements(measurements, allow_hermitian=False):
        if len(measurements) == 0:
            return None
        if len(measurements) == 1 and measurements[0].return_type == "state":
            raise QuantumFunctionError("Not supported")
        if not all(m.return_type == "expval" for m in measurements):
            raise QuantumFunctionError("Adjoint differentiation method does not support expectation return type "
                                       "mixed with other return types")
        for m in measurements:
            obs = m.obs.non_identity_obs if isinstance(m.obs, Q.Tensor) else [m.obs]
            for o in obs:
                if isinstance(o, Q.Projector):
                    raise QuantumFunctionError("Adjoint differentiation method does not support the Projector "
                                               "observable")
                if o.name == "Hermitian" and not allow_hermitian:
                    raise QuantumFunctionError("LightningGPU adjoint differentiation method does not currently "
                                               "support the Hermitian observable")
        return "expval"

    @staticmethod
    def _check_adjdiff_supported_operations(operations):
        # Rot as in the reference (lightning_gpu.py:622-636); CRot and inverted
        # Rot/CRot too, through their exact expansion into one-parameter gates
        for o in operations:
            if o.num_params > 1 and o.name not in ("Rot", "CRot"):
                raise QuantumFunctionError('The %s operation is not supported using the "adjoint" '
                                           "differentiation method" % o.name)

    def adjoint_jacobian(self, tape, starting_state=None, use_device_state=False, split_terms=False):
        """Jacobian [n_observables, n_trainable] by the adjoint method.

        ``split_terms=False`` keeps each Hamiltonian as one observable (one bra
        H|psi> built in one pass per flip mask) instead of the reference's
        one-term split; the summed rows are identical.
        """
        if self.shots is not None:
            warnings.warn("Requested adjoint differentiation to be computed with finite shots. The derivative is "
                          "always exact when using the adjoint differentiation method.", UserWarning)
        self._check_adjdiff_supported_measurements(tape.measurements, self._adjoint_hermitian)
        if len(tape.trainable_params) == 0:
            return np.array(0)
        self._check_adjdiff_supported_operations(tape.operations)
        if starting_state is not None:
            self.syncH2D(np.ravel(starting_state, order="C"))
        elif not use_device_state:
            self.reset()
            self.apply(tape.operations)
        suf = "C64" if self.use_csingle else "C128"
        adj = getattr(self._mod, "AdjointJacobianGPU_" + suf)()
        obs_serialized, obs_offsets = _serialize_observables(tape, self.wire_map, self.use_csingle,
                                                             split_terms=split_terms,
                                                             allow_hermitian=self._adjoint_hermitian)
        ops_serialized, use_sp = _serialize_ops(tape, self.wire_map, self.use_csingle)
        ops_serialized = adj.create_ops_list(*ops_serialized)
        trainable_params = sorted(tape.trainable_params)
        tp_shift, record_tp_rows, all_params = [], [], 0
        for op_idx, tp in enumerate(trainable_params):
            o, _, _ = tape.get_operation(op_idx)
            if not isinstance(o, (Q.BasisState, Q.StatePrep)):
                tp_shift.append(tp)
                record_tp_rows.append(all_params)
            all_params += 1
        # inverted Rot/CRot serialise their parameters reversed: ask for the
        # serialised positions in ascending order, then put the columns back
        pos = _expanded_param_positions(tape)
        mapped = [pos[t] for t in tp_shift]
        order = np.argsort(mapped, kind="stable")
        jac = np.asarray(adj.adjoint_jacobian(self._gpu_state, obs_serialized, ops_serialized,
                                              [mapped[i] for i in order]))
        jac_sorted = jac.reshape(-1, len(tp_shift))
        jac = np.empty_like(jac_sorted)
        jac[:, order] = jac_sorted
        jac_r = np.zeros((len(tape.observables), all_params))
        for idx in range(len(obs_offsets) - 1):
            jac_r[idx, record_tp_rows] = np.sum(jac[obs_offsets[idx]:obs_offsets[idx + 1], :], axis=0)
        return jac_r

    def vjp(self, measurements, dy, starting_state=None, use_device_state=False):
        """Returns a function tape -> dy^T J (reference lightning_gpu.py:771-810)."""
        if self.shots is not None:
            warnings.warn("Requested adjoint differentiation to be computed with finite shots. The derivative is "
                          "always exact when using the adjoint differentiation method.", UserWarning)
        rtype = self._check_adjdiff_supported_measurements(measurements, self._adjoint_hermitian)
        dy = np.asarray(dy)
        if np.allclose(dy, 0) or rtype is None:
            return lambda tape: np.zeros(len(tape.trainable_params))
        if len(dy) != len(measurements):
            raise ValueError("Number of observables in the tape must be the same as the length of dy in the vjp "
                             "method")
        if np.iscomplexobj(dy):
            raise ValueError("The vjp method only works with a real-valued dy when the tape is returning an "
                             "expectation value")
        ham = Q.Hamiltonian(dy, [m.obs for m in measurements])

        def processing_fn(tape):
            if len(tape.trainable_params) == 0:
                return np.array([], dtype=self.C_DTYPE)
            new_tape = Q.QuantumTape(tape.operations, [Q.expval(ham)], tape.trainable_params)
            return self.adjoint_jacobian(new_tape, starting_state, use_device_state)[0]

        return processing_fn

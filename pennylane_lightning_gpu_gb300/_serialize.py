"""Tape serialisation for the adjoint method (reference
pennylane_lightning_gpu/_serialize.py:142-336): observables become the
native ``*ObsGPU_*`` objects, operations become the (names, params, wires,
inverses, matrices) lists of ``OpsStructGPU``; ``Rot`` is expanded into
RZ RY RZ as the reference does (``_serialize.py:311-312``), and, beyond it,
``CRot`` into CRZ CRY CRZ and inverted ``Rot``/``CRot`` into the inverted
factors in reverse order; Hamiltonians are split into one-term Hamiltonians (with offsets)
when ``split_terms`` is set, as the reference does for observable batching.
"""
import numpy as np

from ._native import native
from .ops import Adjoint, BasisState, Hamiltonian, Observable, SparseHamiltonian, StatePrep, Tensor

_PAULI_NAMES = ("PauliX", "PauliY", "PauliZ", "Identity", "Hadamard")


def _suffix(use_csingle):
    return "C64" if use_csingle else "C128"


def _rtype(use_csingle):
    return np.float32 if use_csingle else np.float64


def _ctype(use_csingle):
    return np.complex64 if use_csingle else np.complex128


def _serialize_named_ob(o, wires_map, use_csingle):
    wires = [wires_map[w] for w in o.wires]
    if o.name == "Identity":
        wires = wires[:1]
    return getattr(native(), "NamedObsGPU_" + _suffix(use_csingle))(o.name, wires)


def _serialize_tensor_ob(ob, wires_map, use_csingle, allow_hermitian=False):
    return getattr(native(), "TensorProdObsGPU_" + _suffix(use_csingle))(
        [_serialize_ob(o, wires_map, use_csingle, allow_hermitian=allow_hermitian) for o in ob.obs])


def _serialize_hamiltonian(ob, wires_map, use_csingle, split_terms=True, allow_hermitian=False):
    cls = getattr(native(), "HamiltonianGPU_" + _suffix(use_csingle))
    coeffs = np.array(ob.coeffs).astype(_rtype(use_csingle))
    # a term that is itself a Hamiltonian (a vjp's sum_k dy_k H_k) stays one observable
    terms = [_serialize_ob(t, wires_map, use_csingle, split_terms=False, allow_hermitian=allow_hermitian)
             for t in ob.ops]
    if split_terms:
        return [cls(np.array([c], _rtype(use_csingle)), [t]) for c, t in zip(coeffs, terms)]
    return cls(coeffs, terms)


def _serialize_sparsehamiltonian(ob, wires_map, use_csingle):
    spm = ob.sparse_matrix()
    itype = np.int32 if use_csingle else np.int64
    return getattr(native(), "SparseHamiltonianGPU_" + _suffix(use_csingle))(
        np.array(spm.data).astype(_ctype(use_csingle)), np.array(spm.indices).astype(itype),
        np.array(spm.indptr).astype(itype), [wires_map[w] for w in ob.wires])


def _serialize_hermitian(ob, wires_map, use_csingle):
    return getattr(native(), "HermitianObsGPU_" + _suffix(use_csingle))(
        ob.matrix().astype(_ctype(use_csingle)).ravel(order="C"), [wires_map[w] for w in ob.wires])


def _serialize_ob(ob, wires_map, use_csingle, split_terms=True, allow_hermitian=False):
    if isinstance(ob, Tensor):
        return _serialize_tensor_ob(ob, wires_map, use_csingle, allow_hermitian)
    if isinstance(ob, Hamiltonian):
        return _serialize_hamiltonian(ob, wires_map, use_csingle, split_terms, allow_hermitian)
    if isinstance(ob, SparseHamiltonian):
        return _serialize_sparsehamiltonian(ob, wires_map, use_csingle)
    if ob.name in _PAULI_NAMES:
        return _serialize_named_ob(ob, wires_map, use_csingle)
    if ob.name == "Hermitian":
        if allow_hermitian:
            return _serialize_hermitian(ob, wires_map, use_csingle)
        raise TypeError("Hermitian observables are not currently supported for adjoint differentiation. "
                        "Please use Pauli-words only.")
    raise TypeError("Unknown observable found: %s. Please use Pauli-words only." % (ob,))


def _serialize_observables(tape, wires_map, use_csingle=False, split_terms=True, allow_hermitian=False):
    output, offsets = [], [0]
    for ob in tape.observables:
        ser = _serialize_ob(ob, wires_map, use_csingle, split_terms, allow_hermitian)
        if isinstance(ser, list):
            output.extend(ser)
            offsets.append(offsets[-1] + len(ser))
        else:
            output.append(ser)
            offsets.append(offsets[-1] + 1)
    return output, offsets


_BOUND = {"Identity", "PauliX", "PauliY", "PauliZ", "Hadamard", "S", "T", "RX", "RY", "RZ", "Rot", "PhaseShift",
          "CNOT", "SWAP", "CSWAP", "Toffoli", "CY", "CZ", "CRX", "CRY", "CRZ", "CRot", "ControlledPhaseShift",
          "IsingXX", "IsingYY", "IsingZZ", "MultiRZ", "SingleExcitation", "SingleExcitationMinus",
          "SingleExcitationPlus", "DoubleExcitation", "DoubleExcitationMinus", "DoubleExcitationPlus"}


def _expand_rot(o):
    """Rot(phi, theta, omega) = RZ(omega) RY(theta) RZ(phi), and CRot the same
    product of CRZ/CRY on its (control, target) pair; an inverted one is the
    inverted factors in reverse order, so its parameters come out as
    (omega, theta, phi)."""
    from .ops import op

    phi, theta, omega = o.parameters
    z, y = ("CRZ", "CRY") if o.name == "CRot" else ("RZ", "RY")
    if isinstance(o, Adjoint):
        return [op(z, o.wires, omega).adjoint(), op(y, o.wires, theta).adjoint(), op(z, o.wires, phi).adjoint()]
    return [op(z, o.wires, phi), op(y, o.wires, theta), op(z, o.wires, omega)]


def _expanded_param_positions(tape):
    """pos[q] = index of tape parameter q among the serialised operations'
    parameters. Expansion keeps the count, so pos is the identity except in
    the blocks of inverted Rot/CRot, whose three parameters come out reversed."""
    pos = []
    for o in tape.operations:
        if isinstance(o, (BasisState, StatePrep)):
            continue
        base = len(pos)
        if o.name in ("Rot", "CRot") and isinstance(o, Adjoint):
            pos.extend([base + 2, base + 1, base])
        else:
            pos.extend(range(base, base + len(o.parameters)))
    return pos


def _serialize_ops(tape, wires_map, use_csingle=False):
    names, params, wires, inverses, mats = [], [], [], [], []
    uses_stateprep = False
    for o in tape.operations:
        if isinstance(o, (BasisState, StatePrep)):
            uses_stateprep = True
            continue
        if o.name in ("Rot", "CRot"):
            op_list = _expand_rot(o)
        else:
            op_list = [o]
        for single in op_list:
            is_inverse = isinstance(single, Adjoint)
            names.append(single.name)
            if single.name not in _BOUND:
                params.append(np.zeros(0, _rtype(use_csingle)))
                mats.append(np.asarray(single.matrix(), _ctype(use_csingle)).ravel())
                is_inverse = False  # the matrix is already in inverted form
            else:
                params.append(np.array(single.parameters, _rtype(use_csingle)))
                mats.append(np.zeros(0, _ctype(use_csingle)))
            wires.append([wires_map[w] for w in single.wires])
            inverses.append(is_inverse)
    return (names, params, wires, inverses, mats), uses_stateprep

"""ORACLE — test infrastructure only.

ctypes/numpy front-end of the CPU restatement in ``sv_oracle.hpp``.  The
test-suite, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` use it as the checker; the product never imports it.

Conventions (those of the reference, see ``sv_oracle.hpp``): states are
complex128 arrays of length 2**n, wire ``w`` is index bit ``n-1-w``; matrices
are PennyLane row-major with ``wires[0]`` as the most significant matrix bit.

An *operation* is ``(name, wires, params, inverse, matrix_or_None)``.
An *observable* is ``(is_hamiltonian, [(coeff, [(name, wires, matrix_or_None), ...]), ...])``.
"""
import ctypes
import os

import numpy as np

from . import build as _build

_lib = None

_i64p = ctypes.POINTER(ctypes.c_int64)
_dp = ctypes.POINTER(ctypes.c_double)
_u8p = ctypes.POINTER(ctypes.c_uint8)
_u64p = ctypes.POINTER(ctypes.c_uint64)


class OracleError(RuntimeError):
    pass


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = ctypes.CDLL(path)
        _lib.oracle_last_error.restype = ctypes.c_char_p
    return _lib


def _check(rc):
    if rc != 0:
        raise OracleError(lib().oracle_last_error().decode())


def _ptr(a, t):
    return a.ctypes.data_as(t)


def _as_state(state):
    s = np.ascontiguousarray(state, dtype=np.complex128)
    return s


def _pack_ops(ops):
    names, wire_off, wires, par_off, params, inv, mat_off, mats = [], [0], [], [0], [], [], [0], []
    for op in ops:
        name, w, p, i, m = (list(op) + [None] * 5)[:5]
        names.append(name)
        wires.extend(int(x) for x in w)
        wire_off.append(len(wires))
        params.extend(float(x) for x in (p or []))
        par_off.append(len(params))
        inv.append(1 if i else 0)
        if m is not None:
            mats.extend(np.asarray(m, dtype=np.complex128).ravel())
        mat_off.append(len(mats))
    return dict(
        names="\n".join(names).encode(),
        wire_off=np.array(wire_off, np.int64),
        wires=np.array(wires or [0], np.int64),
        par_off=np.array(par_off, np.int64),
        params=np.array(params or [0.0], np.float64),
        inv=np.array(inv or [0], np.uint8),
        mat_off=np.array(mat_off, np.int64),
        mats=np.array(mats or [0], np.complex128),
        n=len(ops),
    )


def _op_args(p):
    return (
        p["n"],
        p["names"],
        _ptr(p["wire_off"], _i64p),
        _ptr(p["wires"], _i64p),
        _ptr(p["par_off"], _i64p),
        _ptr(p["params"], _dp),
        _ptr(p["inv"], _u8p),
        _ptr(p["mat_off"], _i64p),
        _ptr(p["mats"].view(np.float64), _dp),
    )


def zero_state(n):
    s = np.zeros(1 << n, np.complex128)
    s[0] = 1.0
    return s


def apply_ops(state, ops, n=None):
    """Apply operations to a copy of ``state`` and return it."""
    s = _as_state(state).copy()
    n = n if n is not None else int(np.log2(s.size))
    p = _pack_ops(ops)
    _check(lib().oracle_apply_ops(_ptr(s.view(np.float64), _dp), ctypes.c_int(n), *_op_args(p)))
    return s


def run(n, ops):
    return apply_ops(zero_state(n), ops, n)


def apply_1q_inplace(state, wire, mat):
    """Apply one dense 2x2 gate in place (CPU-baseline single-gate workload)."""
    n = int(np.log2(state.size))
    m = np.ascontiguousarray(mat, dtype=np.complex128).ravel()
    _check(lib().oracle_apply_1q_inplace(_ptr(state.view(np.float64), _dp), ctypes.c_int(n),
                                         ctypes.c_int(wire), _ptr(m.view(np.float64), _dp)))


def set_rot_quirk(on):
    lib().oracle_set_rot_quirk(ctypes.c_int(1 if on else 0))


def expval_matrix(state, mat, wires):
    s = _as_state(state)
    n = int(np.log2(s.size))
    m = np.ascontiguousarray(mat, dtype=np.complex128).ravel()
    w = np.array(wires, np.int64)
    out = np.zeros(2, np.float64)
    _check(lib().oracle_expval_matrix(_ptr(s.view(np.float64), _dp), ctypes.c_int(n), _ptr(w, _i64p),
                                      ctypes.c_int(len(wires)), _ptr(m.view(np.float64), _dp), _ptr(out, _dp)))
    return complex(out[0], out[1])


def expval_pauli_words(state, words, word_wires, coeffs):
    s = _as_state(state)
    n = int(np.log2(s.size))
    off = np.cumsum([0] + [len(w) for w in word_wires]).astype(np.int64)
    flat = np.array([x for w in word_wires for x in w] or [0], np.int64)
    c = np.ascontiguousarray(coeffs, dtype=np.complex128)
    out = np.zeros(1, np.float64)
    _check(lib().oracle_expval_pauli_words(_ptr(s.view(np.float64), _dp), ctypes.c_int(n), ctypes.c_int(len(words)),
                                           "\n".join(words).encode(), _ptr(off, _i64p), _ptr(flat, _i64p),
                                           _ptr(c.view(np.float64), _dp), _ptr(out, _dp)))
    return float(out[0])


def probs(state, wires):
    """Marginal probabilities, output bit k <-> wires[k] (reference 'col-major' order)."""
    s = _as_state(state)
    n = int(np.log2(s.size))
    w = np.array(wires or [0], np.int64)
    out = np.zeros(1 << len(wires), np.float64)
    _check(lib().oracle_probs(_ptr(s.view(np.float64), _dp), ctypes.c_int(n), _ptr(w, _i64p),
                              ctypes.c_int(len(wires)), _ptr(out, _dp)))
    return out


def draws(seed, shots, float_draws=False):
    out = np.zeros(shots, np.float64)
    _check(lib().oracle_draws(ctypes.c_uint64(seed), ctypes.c_int64(shots), ctypes.c_int(1 if float_draws else 0),
                              _ptr(out, _dp)))
    return out


def sample_indices(state, seed, shots, float_draws=False):
    s = _as_state(state)
    n = int(np.log2(s.size))
    out = np.zeros(shots, np.uint64)
    _check(lib().oracle_sample(_ptr(s.view(np.float64), _dp), ctypes.c_int(n), ctypes.c_uint64(seed),
                               ctypes.c_int64(shots), ctypes.c_int(1 if float_draws else 0), _ptr(out, _u64p)))
    return out


def sample_from_draws(state, r):
    s = _as_state(state)
    n = int(np.log2(s.size))
    r = np.ascontiguousarray(r, dtype=np.float64)
    out = np.zeros(r.size, np.uint64)
    _check(lib().oracle_sample_from_draws(_ptr(s.view(np.float64), _dp), ctypes.c_int(n), _ptr(r, _dp),
                                          ctypes.c_int64(r.size), _ptr(out, _u64p)))
    return out


def decode_samples(idx, n):
    """samples[s, n-1-j] = (idx >> j) & 1 (wire 0 is the most significant bit)."""
    idx = np.asarray(idx, np.uint64)
    shifts = np.arange(n - 1, -1, -1, dtype=np.uint64)
    return ((idx[:, None] >> shifts[None, :]) & np.uint64(1)).astype(np.uint64)


def _pack_obs(obs_list):
    term_off, is_ham, coeff, tf_off, fnames, fw_off, fw, fm_off, fm = [0], [], [], [0], [], [0], [], [0], []
    for is_h, terms in obs_list:
        is_ham.append(1 if is_h else 0)
        for c, factors in terms:
            coeff.append(float(c))
            for name, wires, mat in factors:
                fnames.append(name)
                fw.extend(int(x) for x in wires)
                fw_off.append(len(fw))
                if mat is not None:
                    fm.extend(np.asarray(mat, np.complex128).ravel())
                fm_off.append(len(fm))
            tf_off.append(len(fnames))
        term_off.append(len(coeff))
    return dict(
        nobs=len(obs_list),
        term_off=np.array(term_off, np.int64),
        is_ham=np.array(is_ham or [0], np.uint8),
        coeff=np.array(coeff or [0.0], np.float64),
        tf_off=np.array(tf_off, np.int64),
        fnames="\n".join(fnames).encode(),
        fw_off=np.array(fw_off, np.int64),
        fw=np.array(fw or [0], np.int64),
        fm_off=np.array(fm_off, np.int64),
        fm=np.array(fm or [0], np.complex128),
    )


def apply_observable(state, obs):
    s = _as_state(state).copy()
    n = int(np.log2(s.size))
    o = _pack_obs([obs])
    _check(lib().oracle_apply_observable(
        _ptr(s.view(np.float64), _dp), ctypes.c_int(n), ctypes.c_int(int(o["term_off"][1])), _ptr(o["coeff"], _dp),
        ctypes.c_int(int(o["is_ham"][0])), _ptr(o["tf_off"], _i64p), o["fnames"], _ptr(o["fw_off"], _i64p),
        _ptr(o["fw"], _i64p), _ptr(o["fm_off"], _i64p), _ptr(o["fm"].view(np.float64), _dp)))
    return s


def adjoint_jacobian(final_state, ops, obs_list, trainable):
    s = _as_state(final_state)
    n = int(np.log2(s.size))
    p = _pack_ops(ops)
    o = _pack_obs(obs_list)
    tp = np.array(list(trainable) or [0], np.int64)
    jac = np.zeros((len(obs_list), max(len(trainable), 1)), np.float64)
    _check(lib().oracle_adjoint(
        _ptr(s.view(np.float64), _dp), ctypes.c_int(n), *_op_args(p), ctypes.c_int(o["nobs"]),
        _ptr(o["term_off"], _i64p), _ptr(o["is_ham"], _u8p), _ptr(o["coeff"], _dp), _ptr(o["tf_off"], _i64p),
        o["fnames"], _ptr(o["fw_off"], _i64p), _ptr(o["fw"], _i64p), _ptr(o["fm_off"], _i64p),
        _ptr(o["fm"].view(np.float64), _dp), ctypes.c_int64(len(trainable)), _ptr(tp, _i64p), _ptr(jac, _dp)))
    return jac[:, : len(trainable)]


def expval_sparse(state, indptr, indices, data):
    s = _as_state(state)
    n = int(np.log2(s.size))
    off = np.ascontiguousarray(indptr, np.int64)
    cols = np.ascontiguousarray(indices, np.int64)
    vals = np.ascontiguousarray(data, np.complex128)
    out = np.zeros(1, np.float64)
    _check(lib().oracle_expval_sparse(_ptr(s.view(np.float64), _dp), ctypes.c_int(n), _ptr(off, _i64p),
                                      ctypes.c_int64(off.size - 1), _ptr(cols, _i64p),
                                      _ptr(vals.view(np.float64), _dp), _ptr(out, _dp)))
    return float(out[0])

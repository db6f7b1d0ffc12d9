"""Shared helpers of the test-suite (numpy side only)."""
import numpy as np

C128_TOL = 1e-10   # complex128 agreement with the FP64 oracle
C64_TOL = 1e-5     # complex64 agreement with the FP64 oracle


def cls_name(dtype):
    return "LightningGPU_C128" if dtype == "c128" else "LightningGPU_C64"


def np_dtype(dtype):
    return np.complex128 if dtype == "c128" else np.complex64


def tol(dtype):
    return C128_TOL if dtype == "c128" else C64_TOL


def random_unitary(d, rng):
    z = (rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))) / np.sqrt(2)
    q, r = np.linalg.qr(z)
    ph = np.diag(r) / np.abs(np.diag(r))
    return q * ph


def random_hermitian(d, rng):
    a = rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d))
    return (a + a.conj().T) / 2


def random_state(n, rng):
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def make_sv(native, dtype, state):
    """Device state initialised from a host vector."""
    arr = np.ascontiguousarray(state, dtype=np_dtype(dtype))
    return getattr(native, cls_name(dtype))(arr)


def to_oracle_ops(ops):
    return [(o[0], o[1], o[2], o[3], o[4] if len(o) > 4 else None) for o in ops]


def apply_ops(sv, ops):
    """Apply (name, wires, params, inverse[, matrix]) one call each."""
    for o in ops:
        m = o[4] if len(o) > 4 and o[4] is not None else np.zeros(0)
        sv.apply(o[0], list(o[1]), bool(o[3]), list(o[2]), np.asarray(m).ravel())

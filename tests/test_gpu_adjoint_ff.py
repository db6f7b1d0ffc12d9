"""Float-float form of complex128 states through the C ABI: the in-place
conversion lgpu_state_ff, and adjoint blocks that read and leave lambda and
the bras in that form (lgpu_adjoint_block_ff) against the same blocks on
complex128 states (lgpu_adjoint_block); fused gate blocks that pass the
state on in that form (lgpu_apply_fused_block_ff).  Also the Pauli-sum apply that builds
the adjoint's bras from a Hamiltonian (lgpu_apply_pauli_sum: tile passes in
float-float from 16 qubits) against the formula on the host.

Tolerances: the float-float split keeps 48 of the 53 significand bits, so a
round trip changes an amplitude by at most 2^-47 of its magnitude; the two
block paths apply the same float-float arithmetic to the same values and
agree to 1e-13 (states and Jacobian entries).
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LGPU_OK, LGPU_ERR_INVALID_ARG = 0, 1
C64, C128 = 0, 1
FF_IN, FF_OUT = 1, 2


class Step(ctypes.Structure):
    _fields_ = [("tgt", ctypes.c_int32), ("nctrl", ctypes.c_int32), ("ctrl", ctypes.c_int32 * 2),
                ("ctrl_val", ctypes.c_int32 * 2), ("gen_kind", ctypes.c_int32), ("col", ctypes.c_int32),
                ("u", ctypes.c_double * 8), ("g", ctypes.c_double * 8)]


def _lib():
    import pennylane_lightning_gpu_gb300 as pkg

    pkg.build()
    lib = ctypes.CDLL(pkg.library_path())
    vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
    lib.lgpu_context_create.argtypes = [i32, ctypes.POINTER(vp)]
    lib.lgpu_context_destroy.argtypes = [vp]
    lib.lgpu_state_ff.argtypes = [vp, u32, i32, vp]
    block = [vp, vp, ctypes.POINTER(vp), u32, u32, i32, u32, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(Step),
             u32, vp, u32]
    lib.lgpu_adjoint_block.argtypes = block + [vp]
    lib.lgpu_adjoint_block_ff.argtypes = block + [u32, vp]
    return lib


def _state(n, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=1 << n) + 1j * rng.normal(size=1 << n)
    return v / np.linalg.norm(v)


def _mat(m):
    out = (ctypes.c_double * 8)()
    for i, z in enumerate(np.asarray(m, np.complex128).ravel()):
        out[2 * i], out[2 * i + 1] = z.real, z.imag
    return out


def _steps(rng, n):
    """A run of 1-target steps on tile bits 0..10: RY and RX with generators
    (Jacobian columns 0, 1, 2), a CZ as a controlled sign flip, a general
    dense U^dag with a dense generator, and an RZ."""
    def ry(t):
        c, s = np.cos(t / 2), np.sin(t / 2)
        return np.array([[c, s], [-s, c]])

    def rx(t):
        c, s = np.cos(t / 2), np.sin(t / 2)
        return np.array([[c, 1j * s], [1j * s, c]])

    y = np.array([[0, -1j], [1j, 0]])
    x = np.array([[0, 1], [1, 0]])
    q, _ = np.linalg.qr(rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2)))
    h = rng.normal(size=(2, 2)) + 1j * rng.normal(size=(2, 2))
    h = h + h.conj().T
    spec = [(0, [], ry(0.7), y, 0), (3, [], rx(1.9), x, 1), (2, [(1, 1)], np.diag([1, -1]), None, -1),
            (7, [(n - 1, 0)], q, h, 2), (10, [], np.diag([np.exp(-0.4j), np.exp(0.4j)]), None, -1)]
    steps = (Step * len(spec))()
    for s, (tgt, ctrls, u, g, col) in zip(steps, spec):
        s.tgt = tgt
        s.nctrl = len(ctrls)
        for i, (c, v) in enumerate(ctrls):
            s.ctrl[i], s.ctrl_val[i] = c, v
        s.u = _mat(u)
        s.gen_kind = 0 if g is not None else -1
        s.col = col if g is not None else 0
        if g is not None:
            s.g = _mat(g)
    return steps


@pytest.mark.parametrize("n", [12, 20])
def test_state_ff_round_trip(n):
    import torch

    lib = _lib()
    psi = _state(n, 5 + n)
    psi[3] = 0.0  # zero amplitudes stay zero
    d = torch.from_numpy(psi.copy()).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.lgpu_state_ff(d.data_ptr(), n, 1, stream) == LGPU_OK
    f = d.view(torch.float32).reshape(-1, 4).cpu().numpy().astype(np.float64)  # (re.hi, im.hi, re.lo, im.lo)
    re, im = f[:, 0] + f[:, 2], f[:, 1] + f[:, 3]
    assert np.all(np.abs(re - psi.real) <= 2.0 ** -47 * np.abs(psi.real) + 1e-300)
    assert np.all(np.abs(im - psi.imag) <= 2.0 ** -47 * np.abs(psi.imag) + 1e-300)
    assert lib.lgpu_state_ff(d.data_ptr(), n, 0, stream) == LGPU_OK
    back = d.cpu().numpy()
    assert np.max(np.abs(back - psi)) <= 2.0 ** -46 * np.max(np.abs(psi))
    assert back[3] == 0.0


@pytest.mark.parametrize("nbras", [1, 2])
def test_adjoint_block_ff_matches_complex128_blocks(nbras):
    """Two consecutive blocks: complex128 in and out of each, against
    float-float out of the first, in and out of the second, converted back."""
    import torch

    lib = _lib()
    n = 18
    rng = np.random.default_rng(40 + nbras)
    steps = _steps(rng, n)
    tile = (ctypes.c_int32 * 11)(*range(11))
    stream = torch.cuda.current_stream().cuda_stream
    ket0 = _state(n, 1)
    bras0 = [_state(n, 2 + b) for b in range(nbras)]
    ctx = ctypes.c_void_p()
    assert lib.lgpu_context_create(0, ctypes.byref(ctx)) == LGPU_OK
    try:
        results = []
        for ff in (False, True):
            ket = torch.from_numpy(ket0.copy()).cuda()
            bras = [torch.from_numpy(b.copy()).cuda() for b in bras0]
            bptr = (ctypes.c_void_p * nbras)(*[b.data_ptr() for b in bras])
            jac = torch.zeros(2 * 3 * nbras, dtype=torch.float64, device="cuda")
            for blk in range(2):
                out = jac.data_ptr() + blk * 3 * nbras * 8
                if ff:
                    flags = (FF_IN if blk else 0) | FF_OUT
                    st = lib.lgpu_adjoint_block_ff(ctx, ket.data_ptr(), bptr, nbras, n, C128, 11, tile, steps,
                                                   len(steps), out, nbras, flags, stream)
                else:
                    st = lib.lgpu_adjoint_block(ctx, ket.data_ptr(), bptr, nbras, n, C128, 11, tile, steps,
                                                len(steps), out, nbras, stream)
                assert st == LGPU_OK
            if ff:
                assert lib.lgpu_state_ff(ket.data_ptr(), n, 0, stream) == LGPU_OK
                for b in bras:
                    assert lib.lgpu_state_ff(b.data_ptr(), n, 0, stream) == LGPU_OK
            torch.cuda.synchronize()
            results.append((ket.cpu().numpy(), [b.cpu().numpy() for b in bras], jac.cpu().numpy()))
        (k0, b0, j0), (k1, b1, j1) = results
        assert np.max(np.abs(k0 - k1)) < 1e-13
        for x, y in zip(b0, b1):
            assert np.max(np.abs(x - y)) < 1e-13
        assert np.max(np.abs(j0 - j1)) < 1e-13
        assert np.max(np.abs(j0)) > 1e-3  # the generators' overlaps are not all zero
        # complex64 states have no float-float form
        d = torch.zeros(1 << 10, dtype=torch.complex64, device="cuda")
        dp = (ctypes.c_void_p * 1)(d.data_ptr())
        assert lib.lgpu_adjoint_block_ff(ctx, d.data_ptr(), dp, 1, 10, C64, 10,
                                         (ctypes.c_int32 * 10)(*range(10)), steps, len(steps),
                                         jac.data_ptr(), 1, FF_OUT, stream) == LGPU_ERR_INVALID_ARG
    finally:
        lib.lgpu_context_destroy(ctx)


def _pauli_masks(n, words, wires):
    flip, sign, ny = [], [], []
    for word, ws in zip(words, wires):
        f = s = y = 0
        for ch, w in zip(word, ws):
            b = 1 << (n - 1 - w)
            if ch in "XY":
                f |= b
            if ch in "YZ":
                s |= b
            if ch == "Y":
                y += 1
        flip.append(f)
        sign.append(s)
        ny.append(y)
    return flip, sign, ny


@pytest.mark.parametrize("dt,dtype,tol", [(C128, np.complex128, 1e-13), (C64, np.complex64, 2e-5)])
@pytest.mark.parametrize("n", [16, 19])
def test_apply_pauli_sum_tiles_and_wide_words(n, dt, dtype, tol):
    """out = sum_t c_t P_t |in> through lgpu_apply_pauli_sum from 16 qubits:
    words that fit a tile go through the tile passes (float-float for
    complex128), the 9- and 10-flip words through the per-flip-mask passes
    added afterwards; against the formula on the host.  Tolerance: absolute,
    relative to sum_t |c_t| (complex128 1e-13, complex64 2e-5)."""
    import torch

    lib = _lib()
    vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
    lib.lgpu_apply_pauli_sum.argtypes = [vp, vp, u32, i32, u32, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_uint64), ctypes.POINTER(ctypes.c_uint64),
                                         ctypes.POINTER(ctypes.c_uint8), vp]
    rng = np.random.default_rng(90 + n)
    words, wires = ["Z", "ZZ", "XY", "YX", "X", "Y"], [[0], [2, n - 1], [n - 1, n - 2], [0, 1], [n - 9], [3]]
    while len(words) < 40:
        k = int(rng.integers(1, 7))
        wires.append([int(x) for x in rng.choice(n, size=k, replace=False)])
        words.append("".join(rng.choice(list("XYZ"), size=k)))
    words += ["XXXXXXXXX", "YXYXYXYXYX"]
    wires += [list(range(9)), list(range(n - 10, n))]
    coeffs = rng.normal(size=len(words)) + 1j * rng.normal(size=len(words))
    flip, sign, ny = _pauli_masks(n, words, wires)
    psi = _state(n, 7).astype(dtype)
    din = torch.from_numpy(psi.copy()).cuda()
    dout = torch.full_like(din, 3.0)  # overwritten by the first pass
    c = np.ascontiguousarray(np.stack([coeffs.real, coeffs.imag], axis=1).ravel())
    st = lib.lgpu_apply_pauli_sum(din.data_ptr(), dout.data_ptr(), n, dt, len(words),
                                  c.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  (ctypes.c_uint64 * len(words))(*flip), (ctypes.c_uint64 * len(words))(*sign),
                                  (ctypes.c_uint8 * len(words))(*ny), torch.cuda.current_stream().cuda_stream)
    assert st == LGPU_OK
    got = dout.cpu().numpy().astype(np.complex128)
    ref = np.zeros(1 << n, np.complex128)
    idx = np.arange(1 << n, dtype=np.int64)
    p64 = psi.astype(np.complex128)
    for f, s, y, cf in zip(flip, sign, ny, coeffs):
        j = idx ^ f
        par = np.zeros(1 << n, np.int64)
        m = j & s
        while np.any(m):
            par ^= m & 1
            m >>= 1
        ref += cf * (1j ** y) * (1 - 2 * par) * p64[j]
    assert np.max(np.abs(got - ref)) < tol * np.sum(np.abs(coeffs))


class FusedGate(ctypes.Structure):
    _fields_ = [("ntgt", ctypes.c_int32), ("tgt", ctypes.c_int32 * 2), ("nctrl", ctypes.c_int32),
                ("ctrl", ctypes.c_int32 * 4), ("ctrl_val", ctypes.c_int32 * 4), ("m", ctypes.c_double * 32)]


def _fused_block(rng, tile, n, count):
    gates = (FusedGate * count)()
    for g in gates:
        two = rng.random() < 0.25
        t = [int(x) for x in rng.choice(tile, size=2 if two else 1, replace=False)]
        g.ntgt = len(t)
        for i, b in enumerate(t):
            g.tgt[i] = b
        d = 1 << len(t)
        u, _ = np.linalg.qr(rng.normal(size=(d, d)) + 1j * rng.normal(size=(d, d)))
        if rng.random() < 0.3:  # a controlled gate, the control anywhere but on the targets
            c = int(rng.choice([b for b in range(n) if b not in t]))
            g.nctrl, g.ctrl[0], g.ctrl_val[0] = 1, c, int(rng.integers(0, 2))
        for i, z in enumerate(u.ravel()):
            g.m[2 * i], g.m[2 * i + 1] = z.real, z.imag
    return gates


@pytest.mark.parametrize("f64_mode", [1, 0])
def test_fused_blocks_ff_match_complex128_blocks(f64_mode):
    """Three consecutive fused blocks on different tiles: complex128 in and
    out of each, against float-float out of the first, in and out of the
    second, in of the third (the state ends as complex128).  f64_mode 0
    selects the native-FP64 fused kernels, which take complex128 amplitudes:
    the float-float flags then convert the state around the block."""
    import torch

    lib = _lib()
    vp, u32, i32 = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int
    blk = [vp, u32, i32, u32, ctypes.POINTER(ctypes.c_int32), u32, ctypes.POINTER(FusedGate)]
    lib.lgpu_apply_fused_block.argtypes = blk + [vp]
    lib.lgpu_apply_fused_block_ff.argtypes = blk + [u32, vp]
    lib.lgpu_set_f64_mode.argtypes = [i32]
    assert lib.lgpu_set_f64_mode(f64_mode) == LGPU_OK
    try:
        _fused_ff_case(lib, torch)
    finally:
        lib.lgpu_set_f64_mode(1)


def _fused_ff_case(lib, torch):
    n = 19
    rng = np.random.default_rng(17)
    tiles = [list(range(12)), list(range(5)) + list(range(12, 19)), list(range(3)) + [5, 8, 11, 13, 15, 16, 17, 18]]
    blocks = [(t, _fused_block(rng, t, n, 30)) for t in tiles]
    psi = _state(n, 23)
    stream = torch.cuda.current_stream().cuda_stream
    out = []
    for ff in (False, True):
        d = torch.from_numpy(psi.copy()).cuda()
        for i, (t, g) in enumerate(blocks):
            tb = (ctypes.c_int32 * len(t))(*t)
            if ff:
                flags = (FF_IN if i > 0 else 0) | (FF_OUT if i + 1 < len(blocks) else 0)
                st = lib.lgpu_apply_fused_block_ff(d.data_ptr(), n, C128, len(t), tb, len(g), g, flags, stream)
            else:
                st = lib.lgpu_apply_fused_block(d.data_ptr(), n, C128, len(t), tb, len(g), g, stream)
            assert st == LGPU_OK
        out.append(d.cpu().numpy())
    assert np.max(np.abs(out[0] - out[1])) < 1e-13
    assert abs(np.linalg.norm(out[1]) - 1.0) < 1e-12
    # complex64 states have no float-float form
    d64 = torch.zeros(1 << 12, dtype=torch.complex64, device="cuda")
    tb = (ctypes.c_int32 * 12)(*range(12))
    assert lib.lgpu_apply_fused_block_ff(d64.data_ptr(), 12, C64, 12, tb, 1, blocks[0][1], FF_OUT,
                                         stream) == LGPU_ERR_INVALID_ARG

"""Allocation-free inner product ``lgpu_dot_static`` against ``lgpu_dot``,
both called through the C ABI of liblgpu_gb300.so.

The file name keeps it last in collection, so a run of the whole suite
reaches it after every other GPU test; it also passes when run on its own.
The device-reset case runs in a child process of its own, because a reset
ends every allocation of the process's CUDA context.
"""
import ctypes
import os
import subprocess
import sys
import textwrap

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LGPU_OK, LGPU_ERR_INVALID_ARG = 0, 1
C64, C128 = 0, 1


def _lib():
    import pennylane_lightning_gpu_gb300 as pkg

    pkg.build()
    lib = ctypes.CDLL(pkg.library_path())
    vp, u32, i32, dp = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
    lib.lgpu_context_create.argtypes = [i32, ctypes.POINTER(vp)]
    lib.lgpu_context_destroy.argtypes = [vp]
    lib.lgpu_dot.argtypes = [vp, vp, vp, u32, i32, dp, i32, vp]
    lib.lgpu_dot_static.argtypes = [vp, vp, u32, i32, dp, i32, vp]
    lib.lgpu_dot_static_scratch_bytes.restype = ctypes.c_size_t
    lib.lgpu_last_error_string.restype = ctypes.c_char_p
    return lib


def _states(n, dtype, seed):
    rng = np.random.default_rng(seed)
    v = rng.normal(size=(2, 1 << n)) + 1j * rng.normal(size=(2, 1 << n))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    return v.astype(dtype)


@pytest.mark.parametrize("dt,dtype,tol", [(C128, np.complex128, 1e-12), (C64, np.complex64, 1e-5)])
@pytest.mark.parametrize("n", [1, 9, 21])
def test_dot_static_matches_dot_on_consecutive_calls(n, dt, dtype, tol):
    import torch

    lib = _lib()
    host = _states(n, dtype, seed=100 + n)
    a = torch.from_numpy(host[0]).cuda()
    b = torch.from_numpy(host[1]).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    ctx = ctypes.c_void_p()
    assert lib.lgpu_context_create(0, ctypes.byref(ctx)) == LGPU_OK
    try:
        ref = (ctypes.c_double * 2)()
        assert lib.lgpu_dot(ctx, a.data_ptr(), b.data_ptr(), n, dt, ref, 0, stream) == LGPU_OK, \
            lib.lgpu_last_error_string()
        expect = complex(ref[0], ref[1])
        exact = np.vdot(host[0].astype(np.complex128), host[1].astype(np.complex128))
        assert abs(expect - exact) < tol
        for _ in range(2):  # two calls in a row: the arrival counter must come back to zero
            got = (ctypes.c_double * 2)()
            rc = lib.lgpu_dot_static(a.data_ptr(), b.data_ptr(), n, dt, got, 0, stream)
            assert rc == LGPU_OK, lib.lgpu_last_error_string()
            assert abs(complex(got[0], got[1]) - expect) < tol
        # device-side output
        dev = torch.zeros(2, dtype=torch.float64, device="cuda")
        for _ in range(2):
            rc = lib.lgpu_dot_static(a.data_ptr(), b.data_ptr(), n, dt,
                                     ctypes.cast(dev.data_ptr(), ctypes.POINTER(ctypes.c_double)), 1, stream)
            assert rc == LGPU_OK, lib.lgpu_last_error_string()
            torch.cuda.synchronize()
            assert abs(complex(float(dev[0]), float(dev[1])) - expect) < tol
    finally:
        lib.lgpu_context_destroy(ctx)


def test_dot_static_takes_no_device_memory_after_first_call():
    import torch

    lib = _lib()
    n = 20
    host = _states(n, np.complex128, seed=7)
    a = torch.from_numpy(host[0]).cuda()
    b = torch.from_numpy(host[1]).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    out = (ctypes.c_double * 2)()
    assert lib.lgpu_dot_static(a.data_ptr(), b.data_ptr(), n, C128, out, 0, stream) == LGPU_OK
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(5):
        assert lib.lgpu_dot_static(a.data_ptr(), b.data_ptr(), n, C128, out, 0, stream) == LGPU_OK
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    assert abs(complex(out[0], out[1]) - np.vdot(host[0], host[1])) < 1e-12
    assert lib.lgpu_dot_static_scratch_bytes() == 32 << 10


def test_dot_static_rejects_bad_arguments():
    lib = _lib()
    out = (ctypes.c_double * 2)()
    assert lib.lgpu_dot_static(None, None, 4, C128, out, 0, None) == LGPU_ERR_INVALID_ARG
    assert b"null" in lib.lgpu_last_error_string()


def test_dot_static_rejects_null_output():
    import torch

    lib = _lib()
    a = torch.ones(1 << 4, dtype=torch.complex128, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert lib.lgpu_dot_static(a.data_ptr(), a.data_ptr(), 4, C128, None, 0, stream) == LGPU_ERR_INVALID_ARG
    assert b"null" in lib.lgpu_last_error_string()


_RESET_SCRIPT = textwrap.dedent("""
    import ctypes, sys
    import numpy as np
    lib = ctypes.CDLL(sys.argv[1])
    vp, u32, i32, dp = ctypes.c_void_p, ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(ctypes.c_double)
    lib.lgpu_malloc.argtypes = [ctypes.POINTER(vp), ctypes.c_size_t]
    lib.lgpu_free.argtypes = [vp]
    lib.lgpu_memcpy.argtypes = [vp, vp, ctypes.c_size_t, i32, i32, vp]
    lib.lgpu_context_create.argtypes = [i32, ctypes.POINTER(vp)]
    lib.lgpu_context_destroy.argtypes = [vp]
    lib.lgpu_dot.argtypes = [vp, vp, vp, u32, i32, dp, i32, vp]
    lib.lgpu_dot_static.argtypes = [vp, vp, u32, i32, dp, i32, vp]
    lib.lgpu_last_error_string.restype = ctypes.c_char_p
    n = 14
    rng = np.random.default_rng(3)
    host = rng.normal(size=(2, 1 << n)) + 1j * rng.normal(size=(2, 1 << n))
    host = np.ascontiguousarray(host / np.linalg.norm(host, axis=1, keepdims=True))

    def one_round():
        ptrs = []
        for v in host:
            p = vp()
            assert lib.lgpu_malloc(ctypes.byref(p), v.nbytes) == 0, lib.lgpu_last_error_string()
            assert lib.lgpu_memcpy(p, v.ctypes.data, v.nbytes, 0, 0, None) == 0, lib.lgpu_last_error_string()
            ptrs.append(p)
        ctx = vp()
        assert lib.lgpu_context_create(0, ctypes.byref(ctx)) == 0
        ref = (ctypes.c_double * 2)()
        assert lib.lgpu_dot(ctx, ptrs[0], ptrs[1], n, 1, ref, 0, None) == 0, lib.lgpu_last_error_string()
        for _ in range(2):
            got = (ctypes.c_double * 2)()
            rc = lib.lgpu_dot_static(ptrs[0], ptrs[1], n, 1, got, 0, None)
            assert rc == 0, lib.lgpu_last_error_string()
            assert abs(complex(got[0], got[1]) - complex(ref[0], ref[1])) < 1e-12, (got[0], ref[0])
        assert abs(complex(ref[0], ref[1]) - np.vdot(host[0], host[1])) < 1e-12
        lib.lgpu_context_destroy(ctx)
        for p in ptrs:
            assert lib.lgpu_free(p) == 0

    one_round()
    assert lib.lgpu_device_reset() == 0, lib.lgpu_last_error_string()
    one_round()  # the scratch address is looked up again in the new context
    print("reset ok")
""")


def test_dot_static_after_device_reset():
    """lgpu_dot_static, lgpu_device_reset, lgpu_dot_static again, each against
    lgpu_dot, in a child process that owns its own CUDA context."""
    import pennylane_lightning_gpu_gb300 as pkg

    pkg.build()
    r = subprocess.run([sys.executable, "-c", _RESET_SCRIPT, pkg.library_path()], capture_output=True, text=True,
                       timeout=300, env=dict(os.environ))
    assert r.returncode == 0, r.stdout + r.stderr
    assert "reset ok" in r.stdout

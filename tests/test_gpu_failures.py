"""Failure detection without a GPU fault: the bounded device waits give up
and report through the error flag (checked at every synchronisation of the
C++ layer), NaN parameters propagate to NaN results without stalling, and a
waiting serving request can be cancelled while the others complete."""
import ctypes
import time

import numpy as np
import pytest

from pennylane_lightning_gpu_gb300 import serving, workloads

pytestmark = pytest.mark.gpu


def _lib():
    import pennylane_lightning_gpu_gb300 as pkg

    lib = ctypes.CDLL(pkg.library_path())
    lib.lgpu_selftest_bounded_wait.argtypes = [ctypes.c_uint32, ctypes.c_void_p]
    lib.lgpu_device_error.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    lib.lgpu_stream_error.argtypes = [ctypes.c_void_p, ctypes.POINTER(ctypes.c_int), ctypes.c_int]
    lib.lgpu_last_error_string.restype = ctypes.c_char_p
    return lib


def test_bounded_wait_gives_up_and_is_reported(native):
    lib = _lib()
    code = ctypes.c_int(0)
    assert lib.lgpu_device_error(ctypes.byref(code), 1) == 0  # start clean
    t0 = time.perf_counter()
    assert lib.lgpu_selftest_bounded_wait(4096, None) == 0, lib.lgpu_last_error_string()
    assert time.perf_counter() - t0 < 30
    sv = native.LightningGPU_C128(3)
    with pytest.raises(native.PLException, match="timed out"):
        sv.synchronize()  # the C++ layer reads (and clears) the flag at synchronisation
    sv.synchronize()  # cleared: the context is still usable
    sv.Hadamard([0], False, [])
    st = np.asarray(sv.GetState())
    assert abs(st[0] - 2 ** -0.5) < 1e-12 and abs(st[4] - 2 ** -0.5) < 1e-12
    assert lib.lgpu_stream_error(None, ctypes.byref(code), 0) == 0 and code.value == 0
    # the device-wide flag keeps the record until it is reset
    assert lib.lgpu_device_error(ctypes.byref(code), 1) == 0 and code.value == 1
    assert lib.lgpu_device_error(ctypes.byref(code), 0) == 0 and code.value == 0


def test_time_out_is_reported_on_its_own_stream_only(native):
    """A bounded wait that gives up on stream A is raised at A's
    synchronisation and not at a state's on stream B."""
    torch = pytest.importorskip("torch")
    lib = _lib()
    code = ctypes.c_int(0)
    a, b = torch.cuda.Stream(), torch.cuda.Stream()
    for st in (a, b):
        assert lib.lgpu_stream_error(st.cuda_stream, ctypes.byref(code), 1) == 0
    assert lib.lgpu_selftest_bounded_wait(4096, a.cuda_stream) == 0, lib.lgpu_last_error_string()
    assert lib.lgpu_stream_error(b.cuda_stream, ctypes.byref(code), 0) == 0 and code.value == 0
    sv_b = native.LightningGPU_C128(3, native.DevTag(0, b.cuda_stream))
    sv_b.Hadamard([0], False, [])
    sv_b.synchronize()  # nothing timed out on B
    sv_a = native.LightningGPU_C128(3, native.DevTag(0, a.cuda_stream))
    with pytest.raises(native.PLException, match="timed out"):
        sv_a.synchronize()
    sv_a.synchronize()  # A's word was cleared
    assert lib.lgpu_device_error(ctypes.byref(code), 1) == 0 and code.value == 1


def test_selftest_rejects_bad_limit():
    lib = _lib()
    assert lib.lgpu_selftest_bounded_wait(0, None) == 1
    assert lib.lgpu_selftest_bounded_wait(1 << 30, None) == 1


@pytest.mark.parametrize("cls", ["LightningGPU_C128", "LightningGPU_C64"])
def test_nan_parameter_propagates(native, cls):
    sv = getattr(native, cls)(4)
    sv.Hadamard([1], False, [])
    sv.RX([0], False, [float("nan")])
    assert np.isnan(np.asarray(sv.GetState())).any()
    assert np.isnan(np.asarray(sv.Probability([0]))).any()
    ok = getattr(native, cls)(4)  # unaffected
    ok.RX([0], False, [0.4])
    p = np.asarray(ok.Probability([0]))
    assert abs(p[1] - np.sin(0.2) ** 2) < 1e-6


def test_cancel_waiting_request():
    rng = np.random.default_rng(3)
    big = serving.Request(0, 24, workloads.layered_ansatz(24, 10, rng), "expval",
                          obs=workloads.sum_z_hamiltonian_terms(24), arrival=time.perf_counter())
    small = [serving.Request(i, 8, workloads.layered_ansatz(8, 2, rng), "probs", wires=[0, 1],
                             arrival=time.perf_counter()) for i in range(1, 5)]
    srv = serving.CircuitServer(np.complex64, slots=1, micro_batch=False)
    try:
        srv.submit(big)
        for r in small:
            srv.submit(r)
        assert srv.cancel(4)  # still queued behind the big request
        done = srv.drain(timeout=120)
    finally:
        srv.close()
    by_id = {r.rid: r for r in done}
    assert by_id[4].error == "cancelled" and by_id[4].result is None
    for rid in (0, 1, 2, 3):
        assert by_id[rid].error is None and by_id[rid].result is not None
    assert not srv.cancel(0)  # finished requests cannot be cancelled

"""Continuous-batching server: results alone vs in the mix, HBM admission,
latency report.

Tolerances: complex64 expectation values and probabilities 1e-5 (same
kernels alone and in the mix); samples identical for the same seed.
"""
import time

import numpy as np
import pytest

from pennylane_lightning_gpu_gb300 import serving

pytestmark = pytest.mark.gpu


def _trace(count=24, seed=7):
    return serving.make_trace(count, rate=400.0, seed=seed, nmin=6, nmax=18, dmax=5, shots=(200, 500))


def test_results_alone_equal_in_mix():
    m = pytest.importorskip("pennylane_lightning_gpu_gb300")._native.native()
    trace = _trace()
    alone = {r.rid: serving.run_request(m, r, np.complex64) for r in _trace()}
    srv = serving.CircuitServer(np.complex64, slots=6, micro_batch=True, small_n=12)
    try:
        done, makespan = serving.replay(srv, trace)
    finally:
        srv.close()
    assert len(done) == len(trace) and all(r.error is None for r in done)
    for r in done:
        a = alone[r.rid]
        if r.kind == "shots":
            assert np.array_equal(np.asarray(r.result), a)
        else:
            assert np.max(np.abs(np.asarray(r.result) - a)) < 1e-5, (r.kind, r.n)
    rep = serving.report(done, makespan)
    assert rep["completed"] == len(trace) and rep["p99_ms"] >= rep["p50_ms"] > 0


def test_hbm_budget_admission_never_overcommits():
    trace = _trace(16, seed=9)
    biggest = max(r.footprint(8) for r in trace)
    budget = 2 * biggest  # forces admissions to wait for memory
    srv = serving.CircuitServer(np.complex64, slots=8, hbm_budget=budget, micro_batch=False)
    try:
        done, _ = serving.replay(srv, trace)
    finally:
        srv.close()
    assert all(r.error is None for r in done)
    assert srv.max_resident <= budget


def test_oversized_request_rejected_not_hung():
    srv = serving.CircuitServer(np.complex64, slots=2, hbm_budget=1 << 20, micro_batch=False)
    try:
        r = serving.Request(0, 20, [], "expval", obs=[(1.0, "Z", [0])], arrival=time.perf_counter())
        srv.submit(r)
        done = srv.drain(timeout=30)
    finally:
        srv.close()
    assert done and done[0].error is not None and "HBM budget" in done[0].error

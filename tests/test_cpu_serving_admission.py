"""Host-side logic of the continuous-batching server, without a GPU: the
admission policy (HBM footprint budget, oldest fitting request first,
micro-batches of small expectation requests), the seeded request trace and
the latency report."""
import collections

import numpy as np

from pennylane_lightning_gpu_gb300.serving import CircuitServer, Request, make_trace, report


def _server(budget, amp=8, micro=True, small_n=12, max_batch=256):
    # the admission state only; no GPU, streams or dispatcher thread
    s = object.__new__(CircuitServer)
    s.amp, s.budget, s.small_n, s.micro_batch, s.max_batch = amp, budget, small_n, micro, max_batch
    s._waiting = collections.deque()
    s._resident = 0
    s.max_resident = 0
    return s


def _req(rid, n, kind="probs"):
    return Request(rid, n, [], kind)


def test_admission_never_exceeds_the_budget_and_takes_the_oldest_that_fits():
    s = _server(budget=3 * (1 << 20) * 8)  # room for three 20-qubit complex64 states
    for rid, n in enumerate([20, 21, 20, 22, 20, 19]):
        s._waiting.append(_req(rid, n))
    admitted = []
    while True:
        job = s._admit_locked()
        if job is None:
            break
        kind, reqs, need = job
        assert kind == "single" and need == reqs[0].footprint(8)
        assert s._resident <= s.budget
        admitted.append(reqs[0].rid)
    # 20 (8 MiB) and 21 (16 MiB) fill the 24 MiB: none of the others fits now
    assert admitted == [0, 1]
    assert s.max_resident <= s.budget
    # the 21-qubit request finishes: the oldest waiting request that fits goes next
    s._resident -= _req(1, 21).footprint(8)
    kind, reqs, need = s._admit_locked()
    assert reqs[0].rid == 2
    # waiting order is otherwise kept
    assert [r.rid for r in s._waiting] == [3, 4, 5]


def test_small_expectation_requests_are_micro_batched():
    s = _server(budget=1 << 30, small_n=12, max_batch=3)
    s._waiting.extend([_req(0, 10, "expval"), _req(1, 25, "probs"), _req(2, 12, "expval"), _req(3, 8, "expval"),
                       _req(4, 11, "expval"), _req(5, 13, "expval")])
    kind, reqs, need = s._admit_locked()
    assert kind == "batch"
    assert [r.rid for r in reqs] == [0, 2, 3]  # at most max_batch, in arrival order, n <= small_n only
    assert need == sum(r.footprint(8) for r in reqs)
    kind, reqs, _ = s._admit_locked()
    assert kind == "single" and reqs[0].rid == 1  # one small request left: no batch of one
    kind, reqs, _ = s._admit_locked()
    assert kind == "single" and reqs[0].rid == 4
    s2 = _server(budget=1 << 30, micro=False)
    s2._waiting.extend([_req(0, 10, "expval"), _req(1, 10, "expval")])
    assert s2._admit_locked()[0] == "single"


def test_trace_is_seeded_and_shaped_like_the_workload():
    a = make_trace(200, rate=100.0, seed=4)
    b = make_trace(200, rate=100.0, seed=4)
    assert [(r.n, r.kind, len(r.ops), r.shots) for r in a] == [(r.n, r.kind, len(r.ops), r.shots) for r in b]
    arrivals = np.array([r.arrival for r in a])
    assert np.all(np.diff(arrivals) > 0)
    assert 1.0 < arrivals[-1] < 3.5  # 200 requests at 100/s
    ns = np.array([r.n for r in a])
    assert ns.min() >= 8 and ns.max() <= 30
    assert set(r.kind for r in a) == {"expval", "probs", "shots"}
    for r in a:
        if r.kind == "shots":
            assert 1000 <= r.shots <= 10000
        if r.kind == "probs":
            assert r.wires == list(range(min(r.n, 10)))
        if r.kind == "expval":
            assert len(r.obs) == r.n


def test_report_percentiles_and_errors():
    done = []
    for i in range(100):
        r = _req(i, 8)
        r.arrival, r.finish = 0.0, (i + 1) * 1e-3
        done.append(r)
    bad = _req(100, 8)
    bad.arrival, bad.finish, bad.error = 0.0, 1.0, "cancelled"
    out = report(done + [bad], makespan=2.0)
    assert out["requests"] == 101 and out["completed"] == 100 and out["errors"] == 1
    assert abs(out["p50_ms"] - 50.5) < 1e-9
    assert abs(out["p99_ms"] - 99.01) < 1e-9
    assert out["circuits_per_s"] == 50.0


def test_batch_structure_key_ignores_angles_only():
    """Two micro-batches replay the same captured graph exactly when their
    circuits differ only in the angles the batched executor rebuilds on the
    device; the new angles are gathered in circuit and gate order."""
    from pennylane_lightning_gpu_gb300 import workloads
    from pennylane_lightning_gpu_gb300.serving import _structure, _vector_params

    def req(seed, n=6, depth=2, extra=()):
        r = Request(seed, n, workloads.layered_ansatz(n, depth, np.random.default_rng(seed)) + list(extra), "expval")
        r.obs = workloads.sum_z_hamiltonian_terms(n)
        return r

    a, b = req(1), req(2)
    assert _structure(a) == _structure(b)
    assert _structure(a) != _structure(req(1, depth=3))
    assert _structure(a) != _structure(req(1, n=7))
    # a gate whose angle is baked into its matrix is part of the structure
    c, d = req(1, extra=[("MultiRZ", [0, 1], [0.3], False)]), req(2, extra=[("MultiRZ", [0, 1], [0.4], False)])
    assert _structure(c) != _structure(d)
    p = _vector_params([a, b])
    assert p.size == 2 * 2 * 6 * 3
    assert np.allclose(p[:36], [o[2][0] for o in a.ops if o[2]])
    assert np.allclose(p[36:], [o[2][0] for o in b.ops if o[2]])

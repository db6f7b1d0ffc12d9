"""Continuous-batching circuit server.

Requests (a circuit plus one of: expectation value of a Pauli sum,
marginal probabilities, or shots) arrive over time.  The server keeps every
admitted request's state vector resident on the GPU and runs admitted
requests concurrently:

* admission by HBM footprint: a request needs 2^n amplitudes; it is admitted
  when the resident bytes plus its own stay within the budget (free HBM at
  start minus a reserve, or an explicit budget) and a worker slot is free;
* a fixed pool of worker threads, one per slot, each owning a CUDA stream;
  the native calls release the GIL, so the kernels of different requests
  overlap on the device;
* small expectation-value requests (n <= small_n) waiting together are
  micro-batched into one persistent batched launch.  A batch whose circuits
  have the same structure as an earlier batch (gates, wires, observables;
  only rotation angles differ) replays that batch's captured graph with the
  new angles; otherwise the batch is planned and run once without a graph;
* requests that arrive while others run are admitted as soon as memory and
  slots free up (continuous batching, not a FIFO drained one at a time).

Latency = completion time - arrival time; the report gives p50/p99 and
circuits/s.  ``sequential_baseline`` serves the same trace one request at a
time on one stream for comparison.
"""
import collections
import heapq
import threading
import time

import numpy as np

from ._native import native


class Request:
    __slots__ = ("rid", "n", "ops", "kind", "obs", "wires", "shots", "seed", "arrival", "start", "finish",
                 "result", "error", "device_s")

    def __init__(self, rid, n, ops, kind, obs=None, wires=None, shots=0, seed=0, arrival=0.0):
        self.rid, self.n, self.ops, self.kind = rid, n, ops, kind
        self.obs, self.wires, self.shots, self.seed = obs, wires, shots, seed
        self.arrival = arrival
        self.start = self.finish = None
        self.result = None
        self.error = None
        self.device_s = None  # GPU time of the request when served alone (sequential_baseline)

    def footprint(self, amp_bytes):
        return (1 << self.n) * amp_bytes


def _cls(m, dtype):
    return getattr(m, "LightningGPU_C64" if np.dtype(dtype) == np.complex64 else "LightningGPU_C128")


def run_request(m, req, dtype, stream_ptr=None):
    """Execute one request on its own state (optionally on a given stream)."""
    cls = _cls(m, dtype)
    sv = cls(req.n, m.DevTag(0, int(stream_ptr))) if stream_ptr is not None else cls(req.n)
    ops = req.ops
    if ops:
        sv.apply([o[0] for o in ops], [list(o[1]) for o in ops], [bool(o[3]) for o in ops],
                 [list(o[2]) for o in ops])
    if req.kind == "expval":
        words = [t[1] for t in req.obs]
        wires = [list(t[2]) for t in req.obs]
        coeffs = np.array([t[0] for t in req.obs], dtype=dtype)
        out = float(sv.ExpectationValue(words, wires, coeffs))
    elif req.kind == "probs":
        out = np.asarray(sv.Probability(list(req.wires)))
    elif req.kind == "shots":
        sv.setSeed(int(req.seed))
        out = np.asarray(sv.GenerateSampleIndices(int(req.shots), True))
    else:
        raise ValueError("unknown request kind %s" % req.kind)
    sv.synchronize()
    del sv
    return out


# Gates whose parameters the batched executor keeps in its parameter vector
# (rebuilt on the device at every run); every other gate's parameters are part
# of a batch's structure.
_VECTOR_PARAMS = {"RX", "RY", "RZ", "CRX", "CRY", "CRZ", "PhaseShift", "ControlledPhaseShift", "Rot", "CRot",
                  "IsingXX", "IsingYY", "IsingZZ"}


def _structure(req):
    ops = tuple((o[0], tuple(o[1]), bool(o[3]) if len(o) > 3 else False,
                 len(o[2]) if o[0] in _VECTOR_PARAMS else tuple(float(x) for x in o[2])) for o in req.ops)
    obs = tuple((float(c), str(w), tuple(ws)) for c, w, ws in req.obs)
    return (req.n, ops, obs)


def _vector_params(reqs):
    return np.array([float(x) for r in reqs for o in r.ops if o[0] in _VECTOR_PARAMS for x in o[2]], np.float64)


class CircuitServer:
    def __init__(self, dtype=np.complex64, slots=8, hbm_budget=None, reserve_bytes=8 << 30, small_n=12,
                 micro_batch=True, max_batch=256, graph_cache=16):
        import torch

        self.m = native()
        self.dtype = np.dtype(dtype)
        self.amp = 8 if self.dtype == np.complex64 else 16
        free, _ = torch.cuda.mem_get_info()
        self.budget = int(hbm_budget) if hbm_budget is not None else max(int(free - reserve_bytes), 1 << 30)
        self.slots = slots
        self.small_n = small_n
        self.micro_batch = micro_batch
        self.max_batch = max_batch
        self.streams = [torch.cuda.Stream() for _ in range(slots)]
        self._lock = threading.Condition()
        self._waiting = collections.deque()
        self._resident = 0
        self.max_resident = 0
        self._done = []
        self._closed = False
        self._inflight = 0
        # captured batches by structure (least recently used first), and those in use
        self._graphs = collections.OrderedDict()
        self._graph_cache = int(graph_cache)
        self._graphs_busy = set()
        self.graph_hits = 0
        self.batches = 0
        self._workers = [threading.Thread(target=self._worker_loop, args=(slot,), daemon=True)
                         for slot in range(slots)]
        for w in self._workers:
            w.start()

    # ---- client side ------------------------------------------------------
    def submit(self, req):
        need = req.footprint(self.amp)
        if need > self.budget:
            req.error = "request needs %d bytes, more than the HBM budget %d" % (need, self.budget)
            req.finish = time.perf_counter()
            with self._lock:
                self._done.append(req)
                self._lock.notify_all()
            return
        with self._lock:
            self._waiting.append(req)
            self._lock.notify_all()

    def cancel(self, rid):
        """Withdraw a request that has not started: it finishes at once with
        error "cancelled".  Returns False for a running or finished request."""
        with self._lock:
            for r in self._waiting:
                if r.rid == rid:
                    self._waiting.remove(r)
                    r.error = "cancelled"
                    r.finish = time.perf_counter()
                    self._done.append(r)
                    self._lock.notify_all()
                    return True
        return False

    def drain(self, timeout=None):
        """Wait until everything submitted so far has finished."""
        t_end = None if timeout is None else time.perf_counter() + timeout
        with self._lock:
            while self._waiting or self._inflight:
                rem = None if t_end is None else max(0.0, t_end - time.perf_counter())
                if rem == 0.0:
                    raise TimeoutError("server did not drain in time")
                self._lock.wait(timeout=rem)
        return list(self._done)

    def close(self):
        with self._lock:
            self._closed = True
            self._lock.notify_all()
        for w in self._workers:
            w.join(timeout=10)
        self._graphs.clear()

    # ---- workers ------------------------------------------------------------
    def _worker_loop(self, slot):
        while True:
            with self._lock:
                while True:
                    job = self._admit_locked() if self._waiting else None
                    if job is not None:
                        self._inflight += 1
                        break
                    if self._closed and not self._waiting:
                        return
                    self._lock.wait(timeout=0.05)
            self._run_job(slot, job)

    def _admit_locked(self):
        """Pick the next job: a micro-batch of small expval requests or the
        oldest request that fits the memory budget."""
        if self.micro_batch:
            small = [r for r in self._waiting if r.kind == "expval" and r.n <= self.small_n]
            if len(small) >= 2:
                small = small[: self.max_batch]
                need = sum(r.footprint(self.amp) for r in small)
                if self._resident + need <= self.budget:
                    for r in small:
                        self._waiting.remove(r)
                    self._resident += need
                    self.max_resident = max(self.max_resident, self._resident)
                    return ("batch", small, need)
        for r in list(self._waiting):
            need = r.footprint(self.amp)
            if self._resident + need <= self.budget:
                self._waiting.remove(r)
                self._resident += need
                self.max_resident = max(self.max_resident, self._resident)
                return ("single", [r], need)
        return None

    def _run_batch(self, reqs):
        """One micro-batch: replay a captured batch of the same structure with
        the new angles, else plan and run once (and keep it for replays)."""
        from .batched import BatchedExecutor

        reqs = sorted(reqs, key=lambda r: _structure(r))
        key = tuple(_structure(r) for r in reqs)
        with self._lock:
            self.batches += 1
            ex = self._graphs.get(key)
            if ex is not None and key not in self._graphs_busy:
                self._graphs.move_to_end(key)
                self._graphs_busy.add(key)
                self.graph_hits += 1
            else:
                ex = None
        if ex is not None:
            try:
                res = ex.run(_vector_params(reqs))
            finally:
                with self._lock:
                    self._graphs_busy.discard(key)
            return reqs, res
        ex = BatchedExecutor(self.dtype)
        for r in reqs:
            ex.add(r.n, r.ops, r.obs)
        keep = self._graph_cache > 0
        res = ex.prepare(capture=keep).run()
        if keep:
            with self._lock:
                if key not in self._graphs:
                    self._graphs[key] = ex
                    while len(self._graphs) > self._graph_cache:
                        old = next(iter(self._graphs))
                        if old in self._graphs_busy:
                            break
                        self._graphs.pop(old)
        return reqs, res

    def _run_job(self, slot, job):
        kind, reqs, need = job
        t0 = time.perf_counter()
        for r in reqs:
            r.start = t0
        try:
            if kind == "batch":
                reqs, res = self._run_batch(reqs)
                for r, v in zip(reqs, res):
                    r.result = float(v)
            else:
                r = reqs[0]
                r.result = run_request(self.m, r, self.dtype, self.streams[slot].cuda_stream)
        except Exception as e:  # reported per request, the server keeps going
            for r in reqs:
                r.error = repr(e)
        t1 = time.perf_counter()
        with self._lock:
            for r in reqs:
                r.finish = t1
                self._done.append(r)
            self._resident -= need
            self._inflight -= 1
            self._lock.notify_all()


# ---------------------------------------------------------------------------
# load generation and reporting
# ---------------------------------------------------------------------------
def make_trace(count, rate, seed=4, nmin=8, nmax=30, dmin=2, dmax=10, shots=(1000, 10000)):
    """Poisson arrivals (rate per second) of requests with n log-uniform in
    [nmin, nmax], depth uniform in [dmin, dmax] of the layered ansatz, and a
    uniformly chosen measurement: sum_i Z_i, probs on min(n, 10) wires, or a
    number of shots uniform in `shots`."""
    from . import workloads

    rng = np.random.default_rng(seed)
    t = 0.0
    out = []
    for rid in range(count):
        t += float(rng.exponential(1.0 / rate))
        n = int(round(np.exp(rng.uniform(np.log(nmin), np.log(nmax)))))
        depth = int(rng.integers(dmin, dmax + 1))
        ops = workloads.layered_ansatz(n, depth, rng)
        kind = ("expval", "probs", "shots")[int(rng.integers(3))]
        req = Request(rid, n, ops, kind, arrival=t)
        if kind == "expval":
            req.obs = workloads.sum_z_hamiltonian_terms(n)
        elif kind == "probs":
            req.wires = list(range(min(n, 10)))
        else:
            req.shots = int(rng.integers(shots[0], shots[1] + 1))
            req.seed = int(rng.integers(1 << 31))
        out.append(req)
    return out


def replay(server, trace, time_scale=1.0):
    """Submit the trace with its (scaled) inter-arrival times; wait for all."""
    t0 = time.perf_counter()
    for r in trace:
        due = t0 + r.arrival * time_scale
        now = time.perf_counter()
        if due > now:
            time.sleep(due - now)
        r.arrival = time.perf_counter()
        server.submit(r)
    done = server.drain()
    return done, time.perf_counter() - t0


def sequential_baseline(trace, dtype=np.complex64, time_scale=1.0):
    """One request at a time in arrival order on the default stream; a
    request starts at max(its arrival, the previous completion)."""
    import torch

    m = native()
    t0 = time.perf_counter()
    for r in trace:
        due = t0 + r.arrival * time_scale
        now = time.perf_counter()
        if due > now:
            time.sleep(due - now)
        arrival = t0 + r.arrival * time_scale
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        r.start = time.perf_counter()
        ev0.record()
        r.result = run_request(m, r, dtype)
        ev1.record()
        r.finish = time.perf_counter()
        ev1.synchronize()
        r.device_s = ev0.elapsed_time(ev1) / 1e3
        r.arrival = arrival
    return trace, time.perf_counter() - t0


def report(done, makespan):
    lat = np.array([r.finish - r.arrival for r in done if r.error is None])
    ok = len(lat)
    return {"requests": len(done), "completed": ok, "errors": len(done) - ok,
            "p50_ms": float(np.percentile(lat, 50) * 1e3) if ok else None,
            "p99_ms": float(np.percentile(lat, 99) * 1e3) if ok else None,
            "circuits_per_s": ok / makespan if makespan > 0 else None, "makespan_s": makespan}

"""Batched execution of many parameterised circuits in one persistent,
CUDA-graph-captured launch, with a tile/launch-shape autotuner and the plain
one-circuit-at-a-time loop it is compared against.

A circuit is ``(n, ops, observable)`` with ``ops`` a list of
``(name, wires, params, inverse)`` and ``observable`` a list of Pauli terms
``(coeff, word, wires)``; the result of a circuit is <psi|observable|psi>.
"""
import json
import os
import time

import numpy as np

from ._native import native

_CACHE_ENV = "LGPU_AUTOTUNE_CACHE"


def _cls(dtype):
    return "BatchedExecutor_C64" if np.dtype(dtype) == np.complex64 else "BatchedExecutor_C128"


class BatchedExecutor:
    """Owns one native executor: add circuits, prepare once, run many times."""

    def __init__(self, dtype=np.complex128, kmax=0, threads=512, grid=0):
        self.dtype = np.dtype(dtype)
        self._ex = getattr(native(), _cls(dtype))(int(kmax), int(threads), int(grid))
        self.n_circuits = 0

    def add(self, n, ops, observable):
        """Add a circuit; the op tuples and terms are read by the native side
        in one pass (no per-op Python work)."""
        idx = self._ex.add_circuit(int(n), ops, observable)
        self.n_circuits += 1
        return idx

    def add_template(self, n, ops, observable):
        """A circuit structure shared by many parameter sets, lowered and fused
        once; returns its id.  The parameters of the parametric gates in `ops`
        are placeholders (template_num_params(tid) of them, in op order)."""
        return self._ex.add_template(int(n), ops, observable)

    def template_num_params(self, tid):
        return self._ex.template_num_params(int(tid))

    def add_instances(self, tid, params):
        """One circuit per row of `params` (count x template_num_params)."""
        params = np.ascontiguousarray(params, np.float64)
        if params.ndim == 1:
            params = params.reshape(1, -1)
        self.n_circuits += params.shape[0]
        return self._ex.add_instances(int(tid), params)

    def prepare(self, capture=True):
        """Plan and upload.  capture=True also runs the batch once and
        captures the CUDA graph that every run() replays (new parameters go
        through the graph); capture=False enqueues the steps on every run()
        (a batch that runs once)."""
        self._ex.prepare(bool(capture))
        return self

    def run(self, params=None):
        return self._ex.run(None if params is None else np.ascontiguousarray(params, np.float64))

    @property
    def params(self):
        return np.asarray(self._ex.params())

    def stats(self):
        return {"circuits": self._ex.num_circuits(), "gates": self._ex.num_gates(), "blocks": self._ex.num_blocks(),
                "grid": self._ex.grid(), "kmax": self._ex.kmax(), "scratch_bytes": self._ex.scratch_bytes()}


def build_executor(circuits, dtype=np.complex128, kmax=0, threads=512, grid=0):
    ex = BatchedExecutor(dtype, kmax, threads, grid)
    for n, ops, obs in circuits:
        ex.add(n, ops, obs)
    return ex.prepare()


def build_executor_from_templates(templates, dtype=np.complex128, kmax=0, threads=512, grid=0, capture=True):
    """`templates` is a list of ((n, ops, observable), params[count, P]);
    circuits are numbered template by template, row by row."""
    ex = BatchedExecutor(dtype, kmax, threads, grid)
    for (n, ops, obs), params in templates:
        tid = ex.add_template(n, ops, obs)
        ex.add_instances(tid, params)
    return ex.prepare(capture)


def plain_loop(circuits, dtype=np.complex128, fusion=False):
    """The plain per-circuit method: one state vector per circuit, one kernel
    per gate through the drop-in class, then a Pauli-word expectation."""
    m = native()
    cls = getattr(m, "LightningGPU_C64" if np.dtype(dtype) == np.complex64 else "LightningGPU_C128")
    out = np.zeros(len(circuits))
    for i, (n, ops, obs) in enumerate(circuits):
        sv = cls(n)
        if fusion:
            sv.apply([o[0] for o in ops], [list(o[1]) for o in ops], [bool(o[3]) for o in ops],
                     [list(o[2]) for o in ops])
        else:
            for o in ops:
                sv.apply(o[0], list(o[1]), bool(o[3]), list(o[2]), np.zeros(0, dtype))
        words = [t[1] for t in obs]
        wires = [list(t[2]) for t in obs]
        coeffs = np.array([t[0] for t in obs], dtype=dtype)
        out[i] = sv.ExpectationValue(words, wires, coeffs)
    return out


# ---------------------------------------------------------------------------
# autotuner
# ---------------------------------------------------------------------------
def _cache_path():
    return os.environ.get(_CACHE_ENV, os.path.join(os.path.expanduser("~"), ".cache", "lgpu_gb300", "autotune.json"))


def _device_key(dtype, nmin, nmax):
    try:
        import torch

        name = torch.cuda.get_device_name(0)
    except Exception:  # pragma: no cover
        name = "unknown"
    return "%s|%s|n%d-%d" % (name, np.dtype(dtype).name, nmin, nmax)


def autotune(circuits, dtype=np.complex128, sample=256, repeats=3, candidates=None, use_cache=True, seed=0):
    """Pick (kmax, threads) for the batched kernel by timing candidates on a
    seeded sample of the circuits; the choice is cached per GPU model, dtype
    and qubit range."""
    ns = [c[0] for c in circuits]
    key = _device_key(dtype, min(ns), max(ns))
    path = _cache_path()
    cache = {}
    if use_cache and os.path.exists(path):
        try:
            with open(path) as f:
                cache = json.load(f)
        except (OSError, ValueError):
            cache = {}
        if key in cache:
            return cache[key]["kmax"], cache[key]["threads"], cache[key]
    rng = np.random.default_rng(seed)
    idx = rng.choice(len(circuits), size=min(sample, len(circuits)), replace=False)
    sub = [circuits[i] for i in sorted(idx)]
    kmax_max = 13 if np.dtype(dtype) == np.complex128 else 14
    if candidates is None:
        candidates = [(k, t) for k in (kmax_max - 2, kmax_max - 1, kmax_max) for t in (256, 512)]
    timings = {}
    for k, t in candidates:
        ex = build_executor(sub, dtype, kmax=k, threads=t)
        ex.run()
        best = float("inf")
        for _ in range(repeats):
            t0 = time.perf_counter()
            ex.run()
            best = min(best, time.perf_counter() - t0)
        timings["%d/%d" % (k, t)] = best
        del ex
    best_key = min(timings, key=timings.get)
    k, t = (int(x) for x in best_key.split("/"))
    record = {"kmax": k, "threads": t, "timings_s": timings, "sample": len(sub)}
    if use_cache:
        try:
            os.makedirs(os.path.dirname(path), exist_ok=True)
            cache[key] = record
            with open(path, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:  # pragma: no cover - read-only home
            pass
    return k, t, record


def config2_templates(count=4096, nmin=10, nmax=20, lmin=2, lmax=6, seed=2):
    """The batched workload of config2_circuits as templates and parameter
    rows: returns (templates, order) where templates is a list of
    ((n, ops, observable), params[k, P]) for each (n, layers) that occurs and
    order[j] = (template index, row) of circuit j.  The angles are drawn from
    the same seeded stream in the same order, so circuit j is exactly
    config2_circuits(...)[j]."""
    from . import workloads

    rng = np.random.default_rng(seed)
    shapes, rows, order = {}, {}, []
    for _ in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        layers = int(rng.integers(lmin, lmax + 1))
        p = rng.uniform(0, 2 * np.pi, 3 * n * layers)
        key = (n, layers)
        if key not in shapes:
            ops = workloads.layered_ansatz(n, layers, np.random.default_rng(0))
            shapes[key] = (len(shapes), (n, ops, workloads.sum_z_hamiltonian_terms(n)))
            rows[key] = []
        order.append((shapes[key][0], len(rows[key])))
        rows[key].append(p)
    templates = [None] * len(shapes)
    for key, (ti, circ) in shapes.items():
        templates[ti] = (circ, np.array(rows[key]))
    return templates, order


def config2_circuits(count=4096, nmin=10, nmax=20, lmin=2, lmax=6, seed=2):
    """The batched workload: `count` circuits with qubit counts uniform in
    [nmin, nmax], each the layered RX/RY/RZ + CNOT-ring ansatz with
    uniform[lmin, lmax] layers and independent seeded angles; observable
    sum_i Z_i."""
    from . import workloads

    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(nmin, nmax + 1))
        layers = int(rng.integers(lmin, lmax + 1))
        out.append((n, workloads.layered_ansatz(n, layers, rng), workloads.sum_z_hamiltonian_terms(n)))
    return out

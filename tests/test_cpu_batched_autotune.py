"""Host-side logic of the batched executor's autotuner and workload, without a
GPU: the fastest (kmax, threads) candidate wins, the choice is cached per GPU
model, dtype and qubit range, a broken cache file is ignored, and the
batched workload generator is seeded and shaped as specified."""
import json

import numpy as np

from pennylane_lightning_gpu_gb300 import batched


class _Clock:
    def __init__(self):
        self.t = 0.0

    def perf_counter(self):
        return self.t


def _fake_executors(monkeypatch, cost):
    """build_executor returns objects whose run() advances a fake clock by
    cost(kmax, threads); records the candidates tried."""
    clock = _Clock()
    tried = []

    class Ex:
        def __init__(self, k, t):
            self.k, self.t = k, t

        def run(self):
            clock.t += cost(self.k, self.t)

    def build(sub, dtype, kmax=0, threads=512, grid=0):
        tried.append((kmax, threads, len(sub)))
        return Ex(kmax, threads)

    monkeypatch.setattr(batched, "build_executor", build)
    monkeypatch.setattr(batched, "time", clock)
    monkeypatch.setattr(batched, "_device_key", lambda dtype, nmin, nmax: "GPU|%s|n%d-%d" % (
        np.dtype(dtype).name, nmin, nmax))
    return tried


def test_autotune_picks_the_fastest_candidate_and_caches_it(tmp_path, monkeypatch):
    monkeypatch.setenv(batched._CACHE_ENV, str(tmp_path / "tune.json"))
    tried = _fake_executors(monkeypatch, lambda k, t: 1.0 + abs(k - 12) + (0.5 if t == 256 else 0.0))
    circuits = batched.config2_circuits(count=300, seed=7)
    k, t, rec = batched.autotune(circuits, np.complex64, sample=64, repeats=2)
    assert (k, t) == (12, 512)
    assert rec["sample"] == 64 and len(rec["timings_s"]) == 6
    assert {(a, b) for a, b, _ in tried} == {(kk, tt) for kk in (12, 13, 14) for tt in (256, 512)}
    assert all(n == 64 for _, _, n in tried)
    saved = json.loads((tmp_path / "tune.json").read_text())
    assert list(saved.values())[0]["kmax"] == 12
    # second call: from the cache, nothing is timed
    tried.clear()
    assert batched.autotune(circuits, np.complex64)[:2] == (12, 512)
    assert tried == []
    # another dtype is another key: complex128 candidates end at kmax 13
    k2, t2, rec2 = batched.autotune(circuits, np.complex128, sample=32, repeats=1)
    assert (k2, t2) == (12, 512)
    assert {a for a, _, _ in tried} == {11, 12, 13}
    assert len(json.loads((tmp_path / "tune.json").read_text())) == 2


def test_autotune_ignores_a_broken_cache(tmp_path, monkeypatch):
    path = tmp_path / "tune.json"
    path.write_text("{not json")
    monkeypatch.setenv(batched._CACHE_ENV, str(path))
    _fake_executors(monkeypatch, lambda k, t: 2.0 if k == 14 else 3.0)
    circuits = batched.config2_circuits(count=50, seed=1)
    k, t, _ = batched.autotune(circuits, np.complex64, sample=16, repeats=1)
    assert k == 14
    assert json.loads(path.read_text())  # rewritten as valid JSON


def test_config2_workload_shape():
    a = batched.config2_circuits(count=200, seed=2)
    b = batched.config2_circuits(count=200, seed=2)
    assert [(n, len(ops)) for n, ops, _ in a] == [(n, len(ops)) for n, ops, _ in b]
    for n, ops, obs in a:
        assert 10 <= n <= 20
        per_layer = 3 * n + n  # RX, RY, RZ on every wire + CNOT ring
        assert len(ops) % per_layer == 0 and 2 <= len(ops) // per_layer <= 6
        assert len(obs) == n


def test_config2_templates_reproduce_the_circuits():
    """The template form of the 4096-circuit batch (one structure per
    (n, layers), one parameter row per circuit) holds exactly the circuits of
    config2_circuits, angles included."""
    import numpy as np

    from pennylane_lightning_gpu_gb300 import batched

    circuits = batched.config2_circuits(count=300, seed=2)
    templates, order = batched.config2_templates(count=300, seed=2)
    assert len(order) == 300
    assert sum(p.shape[0] for _, p in templates) == 300
    for j, (ti, row) in enumerate(order):
        (n, ops, obs), params = templates[ti]
        n0, ops0, obs0 = circuits[j]
        assert n == n0 and obs == obs0
        assert [(o[0], o[1], o[3]) for o in ops] == [(o[0], o[1], o[3]) for o in ops0]
        assert np.array_equal(params[row], [o[2][0] for o in ops0 if o[2]])

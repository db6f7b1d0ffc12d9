"""The bench's multi-GPU path is one independent replica per rank: the
timed value is all ranks' work over the slowest rank's time.  The rank
helpers run here on two gloo processes (CPU)."""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import torch.distributed as dist

    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    bench._barrier()
    t = bench._max_over_ranks(1.0 + rank)  # rank 1 is the slower replica
    v = bench._replica_value(world, 100.0, t)
    q.put((rank, t, v))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_the_slowest_rank():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in got:
        assert t == 2.0          # max over ranks
        assert v == 2 * 100.0 / 2.0


def test_gate_bytes_follow_the_touched_fraction():
    """Algorithmic bytes per gate: 2S uncontrolled, 2S / 2^c controlled, half
    of that for gates that change only the target-1 amplitudes."""
    import bench

    S = 1 << 20
    assert bench.gate_bytes("RX", S) == 2 * S
    assert bench.gate_bytes("Rot", S) == 2 * S
    assert bench.gate_bytes("RZ", S) == 2 * S
    assert bench.gate_bytes("PhaseShift", S) == S
    assert bench.gate_bytes("CNOT", S) == S
    assert bench.gate_bytes("CRY", S) == S
    assert bench.gate_bytes("CZ", S) == S / 2
    assert bench.gate_bytes("Toffoli", S) == S / 2


def test_distinct_flip_masks():
    import bench

    terms = [(0.5, "ZZ", [0, 1]), (1.0, "Z", [3]), (0.2, "XZ", [2, 0]), (0.1, "YX", [2, 5]),
             (0.3, "XY", [5, 2]), (0.4, "X", [2])]
    # {} (diagonal), {2}, {2, 5}
    assert bench.distinct_flip_masks(terms) == 3
    assert bench.distinct_flip_masks([]) == 0

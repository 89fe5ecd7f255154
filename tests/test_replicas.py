"""Multi-GPU path of the benchmark: independent replicas (one cluster scan per
rank, no data-path collective). The host logic — the slowest rank's time and
the summed work — runs here as two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    # rank r did (r + 2) wavelength-solves in (1 + r) seconds
    times = bench.max_over_ranks([1.0 + rank, 10.0 - rank], world)
    value = bench.replica_value(rank + 2, 1.0 + rank, world)
    out.put((rank, times, value))
    dist.destroy_process_group()


def test_replica_aggregation_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, times, value in res:
        assert times == [2.0, 10.0]          # MAX over ranks
        assert value == pytest.approx(5.0 / 2.0)  # (2 + 3) solves / slowest 2 s


@pytest.mark.parametrize("n,value", [(2, 3.0), (3, 4.0)])
def test_bench_spawns_its_ranks(n, value):
    """`bench.py --gpus N` with no launcher starts N ranks itself (RANK,
    LOCAL_RANK, WORLD_SIZE, local rendezvous); the dry mode runs the ranks'
    gloo aggregation without GPU work: rank r reports r + 1 units in 0.5 (r + 1)
    seconds, so the line carries (1 + .. + N) units over the slowest N / 2 s."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", str(n), "--dry"],
                       capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1  # rank 0 alone prints
    out = json.loads(lines[0])
    assert out["n_gpus"] == n
    assert out["value"] == pytest.approx(value)
    assert out["ms_per_step"] == pytest.approx(500.0 * n)

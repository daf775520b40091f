"""The multi-GPU form is replicas only (independent systems, no data-path
collective): two gloo ranks on CPU check the whole-job timing helpers of
bench.py (slowest rank's time, whole-job rate) and its replica launcher
(`bench.py --gpus N` without torchrun starts N ranks itself)."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local_ms = [12.5, 20.0][rank]
    ms = bench.max_over_ranks(local_ms, world, "cpu")
    out[rank] = (ms, bench.whole_job_rate(16, ms, world))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_max_time_and_rate():
    world = 2
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
        res = dict(out)
    for r in range(world):
        ms, rate = res[r]
        assert ms == 20.0
        assert rate == pytest.approx(2 * 16 * 1000.0 / 20.0)


def test_single_rank_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.0, 1, "cpu") == 7.0
    assert bench.whole_job_rate(16, 8.0, 1) == 2000.0


_WORKER = """
import json, os, sys
sys.path.insert(0, %r)
import torch.distributed as dist
import bench
rank, world, local = bench.dist_env()
dist.init_process_group("gloo")
ms = bench.max_over_ranks([12.5, 20.0][rank], world, "cpu")
if rank == 0:
    print("RESULT " + json.dumps({"n_gpus": world, "ms": ms, "value": bench.whole_job_rate(16, ms, world)}))
dist.barrier()
dist.destroy_process_group()
"""


def test_replica_launcher_two_cpu_ranks(tmp_path, capfd):
    sys.path.insert(0, ROOT)
    import json
    import bench
    worker = tmp_path / "worker.py"
    worker.write_text(_WORKER % ROOT)
    env_saved = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        rc = bench.relaunch_as_replicas(2, str(worker), [])
    finally:
        os.environ.update(env_saved)
    out = capfd.readouterr().out
    assert rc == 0, out
    line = [l for l in out.splitlines() if l.startswith("RESULT ")]
    assert len(line) == 1, out
    res = json.loads(line[0][len("RESULT "):])
    assert res == {"n_gpus": 2, "ms": 20.0, "value": pytest.approx(2 * 16 * 1000.0 / 20.0)}

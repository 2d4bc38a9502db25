"""bench.py's multi-rank logic without a GPU: the slowest rank's time over a world of two gloo
ranks, and the reference arm under two ranks (rank 0 prints the one JSON line, rank 1 exits 0
without work)."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = bench.max_over_ranks(1.5 + rank, dist, torch.device("cpu"))
    q.put((rank, got))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out == {0: 2.5, 1: 2.5}
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.0, None, None) == 3.0


def test_reference_arm_two_ranks():
    oracle = pytest.importorskip("oracle")
    if not os.path.exists(os.path.join(ROOT, "oracle", "_build", "libsvxo.so")):
        pytest.skip("the oracle is not built")
    outs = {}
    for rank in (0, 1):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1")
        r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", "tower",
                            "--steps", "1", "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True,
                           timeout=600)
        assert r.returncode == 0, r.stderr[-2000:]
        outs[rank] = r.stdout.strip()
    assert outs[1] == ""
    line = json.loads(outs[0].splitlines()[-1])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def test_reference_arm_serving_stream():
    """The default workload's reference arm: the serving stream on the host's cores, the same line
    keys as the device arm."""
    pytest.importorskip("oracle")
    if not os.path.exists(os.path.join(ROOT, "oracle", "_build", "libsvxo.so")):
        pytest.skip("the oracle is not built")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3", "--requests", "1000"], cwd=ROOT, capture_output=True, text=True,
                       timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "solves/s" and line["value"] > 0
    assert line["config"]["rtol"] == 1e-6 and line["config"]["timed_requests"] > 0
    assert line["config"]["converged"] == line["config"]["timed_requests"]
    assert line["e2e"]["value"] == line["value"] and line["cpu_baseline"]["kind"] == "port"
    assert line["config"]["requests"] == 1000

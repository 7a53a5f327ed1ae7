"""The N > 1 path of bench.py on CPU: two gloo ranks (127.0.0.1), each with its
own replica timing; the barrier, the max over ranks and the whole-job rate
computed from the slowest rank; the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    ranks = bench.Ranks(world, rank, backend="gloo")
    ranks.barrier()
    ms = 100.0 + 50.0 * rank  # rank 1 is the slower replica
    ms_max = ranks.max(ms)
    out.put((rank, ms_max, bench.whole_job_rate(world, 1000, 10, ms_max), bench.member_seed(rank)))
    ranks.barrier()
    ranks.close()


def test_two_gloo_ranks_time_the_slowest_replica():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as tmp
    ctx = tmp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(2))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [150.0, 150.0]           # max over ranks on both
    assert res[0][2] == res[1][2] == 2 * 1000 * 10 / 0.150  # whole job over the slowest rank
    assert res[0][3] != res[1][3]                          # each rank advances its own member


def test_reference_arm_prints_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""

"""Host side of the multi-GPU bench (independent replicas): two gloo ranks on
the CPU agree on the slowest rank's time and the whole-job rate; the
reference arm's non-zero ranks leave without work or output."""

import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    from euler_kokkos_gb300.replicas import Replicas

    r = Replicas()
    ms = 10.0 + 5.0 * rank  # rank 1 is the slowest
    out.put((rank, r.world, r.max(ms), r.total_rate(1000.0, ms)))
    r.barrier()
    r.close()


def test_two_gloo_ranks_take_the_slowest_time():
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
    assert [r[1] for r in res] == [2, 2]
    assert all(r[2] == 15.0 for r in res)
    # 2 ranks x 1000 units in the slowest rank's 15 ms
    assert all(abs(r[3] - 2000.0 / 0.015) < 1e-6 for r in res)


def test_single_process_is_one_replica():
    sys.path.insert(0, ROOT)
    from euler_kokkos_gb300.replicas import Replicas

    env = {k: os.environ.pop(k) for k in ("RANK", "WORLD_SIZE") if k in os.environ}
    try:
        r = Replicas()
        assert r.world == 1 and r.max(3.5) == 3.5 and r.total_rate(10.0, 2.0) == 5000.0
        r.close()
    finally:
        os.environ.update(env)


def test_reference_arm_nonzero_rank_exits_without_output():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"], env=env,
                       capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert r.returncode == 0 and r.stdout.strip() == ""

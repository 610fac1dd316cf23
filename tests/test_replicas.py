"""Multi-process host logic of bench.py on CPU (gloo, two ranks): the whole job's time is the slowest
replica's, the rate counts every rank's units, and ranks other than 0 of the reference arm exit quietly."""
import os
import socket
import subprocess
import sys

import pytest
import torch
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, ROOT)
    import bench
    torch.distributed.init_process_group("gloo", rank=rank, world_size=world)
    try:
        local_ms = 100.0 + 50.0 * rank
        total = bench.max_over_ranks(local_ms, "cpu")
        torch.distributed.barrier()
        out.put((rank, total, bench.whole_job_rate(1e9, world, 3, total)))
    finally:
        torch.distributed.destroy_process_group()


@pytest.mark.timeout(120)
def test_max_over_ranks_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=90) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    assert [g[1] for g in got] == [150.0, 150.0]  # both ranks see the slowest replica
    assert got[0][2] == pytest.approx(1e9 * 2 * 3 / 0.150)


def test_single_process_is_its_own_max():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, "cpu") == 12.5


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""

"""The N > 1 path of bench.py on CPU: world size 2 over gloo.

bench.py runs one independent plume per rank (replicas: the workload has no
exchange step) and reports the slowest rank's time.  These tests run the
replica seeding and the max-over-ranks reduction in two gloo processes, and
check that the reference arm prints only on rank 0.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "solveit-code_gb300"))
    import bench
    import plume

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    wl = bench.WORKLOADS["fmm_n1m"]
    seed = bench.plume_seed(wl, rank)
    st = plume.make_plume(64, 1e-6, seed)
    slowest = bench.max_over_ranks(1.0 + rank, dist, "cpu")
    gathered = [None] * world
    dist.all_gather_object(gathered, (seed, float(st["x"][0, 2])))
    out.put((rank, slowest, gathered))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_and_max_over_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    out = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    res = [out.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, slowest, gathered in res:
        assert slowest == 2.0                      # max over ranks
        (s0, z0), (s1, z1) = gathered
        assert s0 != s1 and z0 != z1              # each rank its own plume


def test_reference_arm_prints_on_rank0_only(capsys):
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, workload = 1, 0, "direct_n4096"

    bench.run_reference(A, bench.WORKLOADS["direct_n4096"], rank=1, world=2)
    assert capsys.readouterr().out == ""

"""The multi-rank path on CPU: two gloo ranks run independent replicas (here
the CPU oracle stands in for a GPU), the barrier and the max/sum reductions
of poremaps_gb300.replicas combine their timings and work exactly as bench.py
does on GPUs, and each replica's result is the one it computes alone."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), WORLD_SIZE=str(world),
                      RANK=str(rank), LOCAL_RANK=str(rank))
    from oracle.oracle import OracleProblem
    from poremaps_gb300 import synth
    from poremaps_gb300.replicas import Replicas

    rep = Replicas("gloo")
    g = synth.random_solid((10, 8, 12), 0.25, 100 + rank)  # a different sample per rank
    rep.barrier()
    orc = OracleProblem(g, 0, 2)
    orc.iterate(40)
    k = orc.permeability().wk33
    t = 1.0 + rank  # stand-in per-rank times
    out[rank] = (k, rep.max(t), rep.sum(g.size * 40))
    rep.close()


def test_two_gloo_replicas():
    world, port = 2, free_port()
    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(worker, args=(world, port, out), nprocs=world, join=True)
    from oracle.oracle import OracleProblem
    from poremaps_gb300 import synth

    for rank in range(world):
        k, tmax, lups = out[rank]
        g = synth.random_solid((10, 8, 12), 0.25, 100 + rank)
        alone = OracleProblem(g, 0, 2)
        alone.iterate(40)
        assert k == alone.permeability().wk33
        assert tmax == 2.0 and lups == world * 10 * 8 * 12 * 40


def test_reference_arm_other_ranks_exit_without_work(tmp_path):
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference",
                        "--size", "32", "--steps", "1", "--warmup", "1"], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""

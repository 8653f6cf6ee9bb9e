"""Multi-GPU is replicas only (a solve does not shard): N ranks run
independent solves, the bench takes the max elapsed over ranks and counts all
ranks' solves.  Exercise that host logic with two gloo ranks on the CPU, each
running the oracle on its own image."""
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


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), OMP_NUM_THREADS="1")
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import time
    import bench
    from conftest import build_oracle
    from helpers import params, solver
    from ns3d_gb300 import capi, synth
    w, r, local, dist = bench.dist_setup()
    lib = capi.load(build_oracle())
    img, _ = synth.rsa_spheres((10, 8, 9), 2, 0.7, seed=100 + r)
    bench.barrier(dist)
    t = time.perf_counter()
    s = solver(lib, img, params(lib, maxitSIMPLE=5))
    res = s.solve()
    el = time.perf_counter() - t + 0.05 * r   # rank 1 is the slow one
    m = bench.reduce_max(dist, el)
    out[r] = (w, res.K, el, m)
    dist.destroy_process_group()


def test_two_gloo_ranks_max_elapsed():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
    assert all(p.exitcode == 0 for p in procs)
    (w0, k0, e0, m0), (w1, k1, e1, m1) = out[0], out[1]
    assert w0 == w1 == 2
    assert m0 == m1 == max(e0, e1)        # every rank sees the slowest rank's time
    assert k0 > 0 and k1 > 0 and k0 != k1  # independent images, independent solves

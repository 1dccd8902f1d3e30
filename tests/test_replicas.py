"""Replica ranks on the CPU (gloo, world size 2, 127.0.0.1): the benchmark's whole-job aggregation (work summed over
the ranks, the slowest rank's time) and the per-rank batches of the batched workload (rank r solves the batch of
seed r; no collective on the data path)."""

import os
import socket

import numpy as np


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import torch.distributed as tdist

    tdist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        from nuto_gb300 import batch

        vals, sec = bench.aggregate_ranks([rank + 1.0, 10.0 * (rank + 1)], 0.5 + rank, "cpu")
        b, ns, _ = batch.notched_plate_batch(3, seed=rank, n_range=(4, 8))
        q.put((rank, vals, sec, ns.tolist(), int(b.n_dofs)))
    finally:
        tdist.destroy_process_group()


def test_aggregate_single_process_is_identity():
    import bench

    assert bench.aggregate_ranks([3, 4.5], 2.0, "cpu") == ([3.0, 4.5], 2.0)


def test_aggregate_over_two_gloo_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=180) for _ in range(2))
    finally:
        for p in procs:
            p.join(timeout=60)
    assert [p.exitcode for p in procs] == [0, 0]
    for rank, vals, sec, ns, n_dofs in res:
        assert vals == [3.0, 30.0] and sec == 1.5
    assert res[0][3] != res[1][3]  # seed 0 and seed 1: different plates on the two ranks
    assert np.all(np.array(res[0][3] + res[1][3]) >= 4)

"""The multi-GPU path is replicas only: every rank evaluates its own lattice,
with no collective on the data path; the only collective is the max over
ranks of the timing.  Its host logic runs here as two gloo ranks on CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    import torch.distributed as dist

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    import a2c_gb300 as A

    r, w, lr = bench.dist_env()
    t = bench.max_over_ranks(1.0 + rank, w, "cpu")  # rank 1 is the slower one
    X, *_ = A.lattice_fcc(2, pos_std=0.03, seed=bench.replica_seed(bench.WORKLOAD["seed"], r))
    out[rank] = (r, w, t, float(X[:12].sum()))
    dist.destroy_process_group()


def test_two_rank_replicas_gloo():
    world = 2
    port = _free_port()
    mgr = mp.get_context("spawn").Manager()
    out = mgr.dict()
    mp.start_processes(_rank_main, args=(world, port, out), nprocs=world, start_method="spawn", join=True)
    (r0, w0, t0, s0), (r1, w1, t1, s1) = out[0], out[1]
    assert (r0, r1, w0, w1) == (0, 1, 2, 2)
    assert t0 == t1 == 2.0  # both ranks see the slowest rank's time
    assert s0 != s1  # independent replicas
    import bench

    assert bench.whole_job_value(1000, 10, 2, 2.0) == 2 * 1000 * 10 / 2.0

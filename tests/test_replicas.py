"""Several GPUs run independent replicas (bench.py --gpus N under torchrun):
each rank takes its own seeds, and rank 0 reports the summed events over
the slowest rank's time.  This checks that aggregation with two gloo ranks
on the CPU, the oracle standing in for each rank's device work."""
import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank),
                      MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    import bench
    import oracle
    from spatialpy_gb300 import scenario as S
    w, r, _, pg = bench.dist_setup()
    sc = S.config_birth_death_2d(n=6, t_end=2.0, num_points=3)
    seeds = np.arange(4, dtype=np.uint64) + bench.SEED0 + np.uint64(r * 1000003)
    _, ev, _, _ = oracle.nsm_ensemble(sc, seeds, 0, 1, want_counts=False)
    bench.barrier(pg)
    total = bench.sum_over_ranks(pg, float(ev.sum()))
    slowest = bench.max_over_ranks(pg, float(r + 1))
    out[rank] = (w, float(ev.sum()), total, slowest)
    pg.destroy_process_group()


def test_two_replicas_sum_events_and_take_the_slowest_rank():
    import oracle
    from spatialpy_gb300 import scenario as S
    oracle.build()
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
        res = dict(out)
    assert res[0][0] == 2 and res[1][0] == 2
    assert res[0][2] == res[1][2] == res[0][1] + res[1][1]
    assert res[0][3] == res[1][3] == 2.0
    # the two ranks' seeds differ, and together equal a one-process run
    sc = S.config_birth_death_2d(n=6, t_end=2.0, num_points=3)
    import bench
    seeds = np.concatenate([np.arange(4, dtype=np.uint64) + bench.SEED0 + np.uint64(r * 1000003)
                            for r in range(2)])
    _, ev, _, _ = oracle.nsm_ensemble(sc, seeds, 0, 1, want_counts=False)
    assert float(ev.sum()) == res[0][2]

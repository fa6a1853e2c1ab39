"""The multi-GPU form of bench.py (one process per GPU under torchrun, every rank its own
ensemble, no data exchange): rank environment and the job aggregation (max of the timed
milliseconds, sum of the nodes) on two gloo ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as tdist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), LOCAL_RANK=str(rank),
                      WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench

    r, lr, ws = bench.dist_env()
    tdist.init_process_group("gloo", rank=r, world_size=ws)
    # rank k "took" 10 + k ms over its own ensemble of 1000 * (k + 1) nodes
    ms, nodes = bench.reduce_over_ranks(tdist, 10.0 + r, 1000 * (r + 1), "cpu")
    tdist.barrier()
    tdist.destroy_process_group()
    out[rank] = (r, lr, ws, ms, nodes)


def test_two_gloo_ranks_aggregate_max_time_and_total_nodes():
    world = 2
    out = mp.Manager().dict()
    mp.spawn(_rank_main, args=(world, _free_port(), out), nprocs=world, join=True)
    for rank in range(world):
        r, lr, ws, ms, nodes = out[rank]
        assert (r, lr, ws) == (rank, rank, world)
        assert ms == 11.0 and nodes == 3000


def test_single_process_needs_no_collective():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.reduce_over_ranks(None, 7.5, 123, "cpu") == (7.5, 123)


def test_ranks_run_different_ensembles_of_the_same_kind(monkeypatch):
    """Weak scaling: rank k builds the ensemble of the same kind from its own seed."""
    sys.path.insert(0, ROOT)
    import bench
    from perigrain_gb300 import setups

    seen = []
    monkeypatch.setattr(setups, "workload", lambda k, **kw: seen.append((k, kw)) or setups.collision_ensemble(
        n_inst=4, **kw))
    s0, spec0 = bench.build_workload(3, 0)
    s1, spec1 = bench.build_workload(3, 1)
    assert seen[0][1]["seed"] != seen[1][1]["seed"] and spec0 is spec1
    assert s0.n_instances == s1.n_instances == 4
    assert s0.n_nodes != s1.n_nodes or (s0.pos != s1.pos).any()

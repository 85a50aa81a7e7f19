"""Multi-GPU runs are independent replicas (one solve per rank, no collective on
the data path); the host-side logic -- max-over-ranks timing and the whole-job
value -- runs here on CPU as two gloo ranks."""
import os
import socket

import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local = 1.0 + rank                     # rank 1 is the slower replica
    secs = bench.replica_seconds(local, dist, "cpu")
    out[rank] = (secs, bench.replica_value(1000, 10, world, secs))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_take_max_time_and_sum_work():
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    assert res[0] == res[1] == (2.0, 2 * 1000 * 10 / 2.0)


def test_single_rank_is_local_time():
    import bench
    assert bench.replica_seconds(3.5) == 3.5
    assert bench.replica_value(10, 5, 1, 2.0) == 25.0


def _shard_rank(rank, world, port, out):
    import torch.distributed as dist
    import bench
    from se2dr_fork_gb300 import spec as S
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    shard = S.ensemble_shard(3, rank, seed=5)
    dof = sum(2 * sp.nnodes for sp in shard)
    out[rank] = ([(sp.mx, sp.my, sp.p, sp.sources[0].x) for sp in shard], dof, bench.job_sum(dof, dist, "cpu"),
                 bench.replica_seconds(1.0 + rank, dist, "cpu"))
    dist.barrier()
    dist.destroy_process_group()


def test_ensemble_shards_are_disjoint_blocks_and_work_sums():
    """Multi-GPU ensembles: rank r runs draws r*n ... (r+1)*n-1 of the ensemble distribution (no
    exchange); the job's work is the sum over ranks and its time the slowest rank's."""
    from se2dr_fork_gb300 import spec as S
    world = 2
    port = _free_port()
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_shard_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    both = S.ensemble(6, seed=5)
    ref = [(sp.mx, sp.my, sp.p, sp.sources[0].x) for sp in both]
    assert res[0][0] + res[1][0] == ref
    assert res[0][2] == res[1][2] == res[0][1] + res[1][1]
    assert res[0][3] == res[1][3] == 2.0

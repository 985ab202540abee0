"""bench.py --gpus N runs one independent replica per GPU (the PFEM-2 step does not
shard); the job's ms per step is the slowest replica's.  The reduction across ranks is
checked here with two gloo ranks on the CPU."""
import os
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _rank(rank, world, port, values, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    out[rank] = bench.replica_max(values[rank], "cpu")
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_replica_max_over_gloo_ranks(world):
    values = [161.5 + 3.0 * r for r in range(world)][::-1]
    with mp.Manager() as mgr:
        out = mgr.dict()
        port = 29500 + os.getpid() % 1000 + world
        mp.start_processes(_rank, args=(world, port, values, out), nprocs=world, join=True, start_method="spawn")
        assert [out[r] for r in range(world)] == [max(values)] * world

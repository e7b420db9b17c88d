"""The N > 1 path of the benchmark as gloo ranks on the CPU: each rank traces its
own disjoint flight range (here with the oracle), the records of the ranks
together equal one batch over the whole range, and the timing reductions give the
slowest rank's time and the summed work."""
import os
import tempfile

import numpy as np
import pytest

from gpis_extend_gb300 import replicas, workloads
from oracle import oracle

N = 192


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    desc = workloads.sphere_medium()
    prim = workloads.sphere_flights(N, desc, index_offset=replicas.flight_range(N, rank))
    rec = oracle.trace_flights(desc, prim, n_threads=1)
    np.save(os.path.join(out_dir, f"rec{rank}.npy"), rec)
    red = replicas.Reducer(dist)
    t = red.max(1.0 + rank)
    total = red.sum(N)
    rate = red.throughput(N, 1.0 + rank)
    red.barrier()
    np.save(os.path.join(out_dir, f"red{rank}.npy"), np.array([t, total, rate]))
    dist.destroy_process_group()


def test_gloo_replicas_trace_disjoint_ranges():
    mp = pytest.importorskip("torch.multiprocessing")
    pytest.importorskip("torch.distributed")
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    world = 2
    with tempfile.TemporaryDirectory() as d:
        mp.start_processes(_rank, args=(world, port, d), nprocs=world, start_method="spawn", join=True)
        recs = [np.load(os.path.join(d, f"rec{r}.npy")) for r in range(world)]
        reds = [np.load(os.path.join(d, f"red{r}.npy")) for r in range(world)]
    desc = workloads.sphere_medium()
    whole = oracle.trace_flights(desc, workloads.sphere_flights(world * N, desc), n_threads=1)
    assert np.array_equal(np.concatenate(recs).view(np.uint32), whole.view(np.uint32))
    for t, total, rate in reds:
        assert t == 2.0 and total == world * N and rate == world * N / 2.0

"""The multi-GPU path of bench.py on CPU: two gloo ranks. The path shards by
spectrum with no exchange (independent replicas, one seeded batch per rank);
the only collective is the max-reduction of the step times, and the job's
throughput counts every rank's evaluations."""
import os
import socket
import sys

import numpy as np
import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    import bench
    from coffe_gb300 import workloads

    torch.distributed.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}",
                                         rank=rank, world_size=world)
    try:
        # per-rank timings: rank r took (r + 1) x the base times
        got = bench.reduce_over_ranks(torch, [0.5 * (rank + 1), 2.0 * (rank + 1), 1e-3 * (rank + 1)],
                                      world, torch.device("cpu"))
        batch = workloads.cfg3(n_spectra=2, seed=workloads.CFG3_SEED + rank)
        # the reference arm does its work on rank 0 only
        idle = bench.reference_arm(None, rank, world) if rank != 0 else None
        np.savez(os.path.join(out_dir, f"rank{rank}.npz"), got=np.array(got), pk=batch.pk,
                 n_evals=batch.n_evals, idle=idle is None)
    finally:
        torch.distributed.destroy_process_group()


def test_two_rank_replicas(tmp_path):
    world = 2
    torch.multiprocessing.spawn(_rank_main, args=(world, _free_port(), str(tmp_path)), nprocs=world,
                                join=True)
    r0, r1 = (np.load(tmp_path / f"rank{r}.npz") for r in range(world))
    # every rank holds the maximum over the ranks
    assert np.allclose(r0["got"], [1.0, 4.0, 2e-3]) and np.allclose(r1["got"], r0["got"])
    # independent replicas: different seeded spectra per rank, same shapes
    assert r0["pk"].shape == r1["pk"].shape and not np.allclose(r0["pk"], r1["pk"])
    assert bool(r1["idle"])
    import bench

    # whole-job throughput: both ranks' evaluations over the slowest rank's time
    n = int(r0["n_evals"])
    assert bench.job_throughput(n, 10, world, 2.0) == pytest.approx(n * 10 * 2 / 2.0)

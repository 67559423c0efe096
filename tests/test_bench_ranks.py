"""The multi-process side of bench.py on CPU: two gloo ranks, as torchrun would start them
for `bench.py --gpus 2`. The engine does not shard a force evaluation (every rank runs its
own replica of the workload, with no collective on the data path), so what N > 1 adds is
host logic: the step time is the maximum over ranks on every rank, the job's rate is the
ranks' units over that time, and the reference arm runs on rank 0 alone."""
import json
import os
import socket

import pytest

from conftest import ROOT


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out_dir):
    import sys
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # the slowest rank sets the step time; each rank's own figure differs
        ms = bench.max_over_ranks(dist, 1.25 + rank, "cpu")
        e2e = bench.max_over_ranks(dist, 3.0 - rank, "cpu")
        rate = bench.job_rate(world, 1000, ms)
        # the reference arm: ranks other than 0 leave at once, with status 0 and no output
        ref = bench.run_reference(None, rank) if rank != 0 else None
        dist.barrier()
    finally:
        dist.destroy_process_group()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"ms": ms, "e2e": e2e, "rate": rate, "ref": ref}, f)


def test_two_gloo_ranks(tmp_path):
    mp = pytest.importorskip("torch.multiprocessing")
    world = 2
    mp.start_processes(rank_main, args=(world, free_port(), str(tmp_path)), nprocs=world, join=True,
                       start_method="spawn")
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(world)]
    for r in res:
        assert r["ms"] == 2.25 and r["e2e"] == 3.0
        assert r["rate"] == pytest.approx(world * 1000 / 2.25e-3)
    assert res[1]["ref"] == 0


def test_single_process_is_unchanged():
    import bench
    assert bench.max_over_ranks(None, 1.5, "cpu") == 1.5
    assert bench.job_rate(1, 500, 2.0) == pytest.approx(2.5e5)

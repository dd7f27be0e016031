"""Multi-process harness of the benchmark, on CPU with the gloo backend (world size 2).

The step has no exchange between GPUs: at N > 1 every rank steps an independent replica
(its own seeded system), the job time is the slowest rank's, and the reference arm runs on
rank 0 only.  These tests cover that host logic without a GPU.
"""
import io
import os
import socket
import contextlib

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, ws, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import bench

    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        got_ws, got_rank, got_local = bench.dist_setup()
        t_max = bench.max_over_ranks(0.25 * (rank + 1), got_ws, torch.device("cpu"))
        buf = io.StringIO()
        args = type("A", (), {"n": 1024, "grid": 8, "steps": 1, "gpus": ws,
                              "ref_sample_boxes": 4})()
        if rank != 0:  # rank 0 would time the CPU reference; only the idle ranks are checked
            with contextlib.redirect_stdout(buf):
                r = bench.run_reference(args, got_ws, got_rank)
            assert r is None
        with open(os.path.join(out_dir, f"rank{rank}.txt"), "w") as f:
            f.write(f"{got_ws} {got_rank} {got_local} {t_max!r} {bench.replica_seed(rank)} "
                    f"{len(buf.getvalue())}\n")
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_gloo(tmp_path):
    ws = 2
    mp.start_processes(_worker, args=(ws, _free_port(), str(tmp_path)), nprocs=ws,
                       join=True, start_method="spawn")
    rows = [open(tmp_path / f"rank{r}.txt").read().split() for r in range(ws)]
    seeds = set()
    for r, row in enumerate(rows):
        got_ws, got_rank, got_local, t_max, seed, printed = row
        assert (int(got_ws), int(got_rank), int(got_local)) == (ws, r, r)
        assert float(t_max) == pytest.approx(0.5)  # every rank sees the slowest rank's time
        seeds.add(int(seed))
        if r != 0:
            assert int(printed) == 0  # non-zero ranks print nothing in the reference arm
    assert len(seeds) == ws  # replicas step different systems


def test_single_rank_time_passthrough():
    import bench

    assert bench.max_over_ranks(1.5, 1, torch.device("cpu")) == 1.5

"""The box-slab decomposition over ranks (barneshut/gb300/slabs.py), on CPU ranks with the gloo
backend: each rank keeps the particles of its own boxes, exchanges particles that changed rank,
the leaf moments and the near-field halo, and evaluates its own particles with the oracle.  After
the steps, the ranks' particles gathered by particle id equal a single-rank run of the same oracle
bit for bit: every sum runs in the same order (boxes' particles in particle-id order on every
rank, the whole grid's moments an exact sum of per-rank moments).

Host logic only; the multi-GPU path has not run on hardware (one GPU per machine in this build).
"""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

N, G, STEPS, DT = 3000, 16, 2, 1e-5
CASES = {
    # name: (theta, group_dim, eps2, cutoff, dense_min, quad_min)
    "flat_reference": (0.0, 1, 0.0, 1e-5, 0, 0),
    "theta_refined": (0.5, 2, 1e-6, 0.0, 16, 48),
}


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _system():
    from barneshut.gb300 import workloads

    x, y, m, vx, vy = workloads.cluster_mixture(N, seed=91)
    vx = np.random.default_rng(92).normal(0, 0.3, N)
    vy = np.random.default_rng(93).normal(0, 0.3, N)
    return x, y, m, vx, vy


def _single_rank(case):
    from oracle import oracle

    theta, TG, eps2, cut, dmin, qmin = CASES[case]
    x, y, m, vx, vy = (a.copy() for a in _system())
    for _ in range(STEPS):
        ax, ay, _, _ = oracle.theta_evaluate(x, y, m, G, TG=TG, theta=theta, eps2=eps2, cutoff=cut,
                                             dense_min=dmin, quad_min=qmin)
        x, y, vx, vy = oracle.tick(x, y, vx, vy, ax, ay, DT)
    return np.column_stack([x, y, m, vx, vy])


def _worker(rank, ws, port, case, out_dir):
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "barnes-hut_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        from barneshut.gb300 import slabs
        from oracle import oracle

        theta, TG, eps2, cut, dmin, qmin = CASES[case]
        x, y, m, vx, vy = _system()
        pid = np.arange(N, dtype=np.float64)
        # start from an arbitrary split (particle-id chunks), as the reference does
        lo, hi = rank * N // ws, (rank + 1) * N // ws
        state = np.column_stack([x, y, m, vx, vy, pid])[lo:hi]
        comm = slabs.SlabComm("cpu")
        sysl = slabs.SlabSystem(state, G, comm, theta=theta, group_dim=TG)

        def evaluator(xa, ya, ma, targets, bb, leaf, extents):
            ax, ay, _, _ = oracle.theta_evaluate_part(xa, ya, ma, G, bb, leaf, targets, TG=TG,
                                                      theta=theta, eps2=eps2, cutoff=cut,
                                                      dense_min=dmin, quad_min=qmin)
            return ax, ay

        for _ in range(STEPS):
            sysl.create_tree()
            sysl.summarize(oracle.leaf_moments)
            sysl.evaluate(evaluator)
            sysl.timestep(DT)
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), sysl.state)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("ws", [2, 3])
def test_slab_step_equals_single_rank(tmp_path, case, ws, oracle_mod):
    # (the oracle is built once here, before the ranks load it)
    mp.start_processes(_worker, args=(ws, _free_port(), case, str(tmp_path)), nprocs=ws,
                       join=True, start_method="spawn")
    parts = [np.load(tmp_path / f"rank{r}.npy") for r in range(ws)]
    assert all(len(p) > 0 for p in parts)
    allp = np.concatenate(parts)
    pid = allp[:, 5].astype(np.int64)
    assert np.array_equal(np.sort(pid), np.arange(N))  # every particle on exactly one rank
    got = allp[np.argsort(pid)][:, :5]
    ref = _single_rank(case)
    np.testing.assert_array_equal(got, ref)


def test_partition_and_halo_host_logic():
    from barneshut.gb300 import slabs

    r = slabs.box_ranges(16, 3)
    assert r == [(0, 86), (86, 171), (171, 256)]  # np.array_split of 256 boxes
    assert [len(a) for a in np.array_split(np.arange(256), 3)] == [b - a for a, b in r]
    own = slabs.owner_of_boxes([0, 85, 86, 170, 171, 255], r)
    assert list(own) == [0, 0, 1, 1, 2, 2]
    # reach 1 around boxes 86..170 of a 16 x 16 grid: the adjacent boxes of ranks 0 and 2
    h = slabs.halo_boxes(16, 86, 171, 1)
    assert not np.any((h >= 86) & (h < 171))
    gx, gy = h // 16, h % 16
    own_x, own_y = np.arange(86, 171) // 16, np.arange(86, 171) % 16
    for a, b in zip(gx, gy):
        assert np.min(np.maximum(np.abs(own_x - a), np.abs(own_y - b))) == 1
    assert slabs.halo_reach(0.0, 4) == 1
    assert slabs.halo_reach(0.5, 2) == 1 + 2 + 2
    bb = slabs.square_box(0.0, 0.1, 0.5, 0.3, 8)
    np.testing.assert_array_equal(bb, [0.0, 0.1, 0.5, 0.3 + ((0.5 - 0.0) - (0.3 - 0.1)), 0.5 / 8])

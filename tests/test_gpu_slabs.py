"""The box-slab step with the CUDA evaluator (barneshut/gb300/slabs.py PlanSlab): two ranks as
two processes on the one GPU of this machine, exchanging over gloo on the host (their kernels
never wait on each other).  Each rank runs a plan over its own and halo particles with the
whole system's grid (bh_set_grid) and far field (bh_set_leaf_moments).

Tolerances, against one plan over the whole system on the same GPU (same kernels, same
opening rule): accelerations of every particle within relative RMS 1e-6 (the FP32 per-warp
partial sums of the leaf moments start at other particle offsets on a rank) and positions
after the steps within 1e-9 of the unit box; and against the FP64 oracle, relative RMS 1e-5.
"""
import os
import socket

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")

N, G, STEPS, DT = 20000, 32, 2, 1e-5
CASES = {
    # name: (theta, group_dim, softening, cutoff, dense_min, quad_min)
    "theta_stream": (0.5, 2, 1e-3, 0.0, 16, 48),
    "flat_reference": (0.0, 1, 0.0, 1e-5, 0, -1),
}


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _system():
    from barneshut.gb300 import workloads

    x, y, m, _, _ = workloads.cluster_mixture(N, seed=95)
    vx = np.random.default_rng(96).normal(0, 0.3, N)
    vy = np.random.default_rng(97).normal(0, 0.3, N)
    return x, y, m, vx, vy


def _params(case):
    from barneshut.gb300 import native

    theta, TG, eps, cut, dmin, qmin = CASES[case]
    return native.make_params(1.0, DT, eps, cut, theta, TG, native.BH_PREC_FP32_KAHAN,
                              dense_min=dmin, quad_min=qmin)


def _worker(rank, ws, port, case, out_dir):
    import sys

    import torch.distributed as dist

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for p in (root, os.path.join(root, "barnes-hut_gb300")):
        if p not in sys.path:
            sys.path.insert(0, p)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        from barneshut.gb300 import slabs

        theta, TG = CASES[case][:2]
        x, y, m, vx, vy = _system()
        pid = np.arange(N, dtype=np.float64)
        lo, hi = rank * N // ws, (rank + 1) * N // ws
        state = np.column_stack([x, y, m, vx, vy, pid])[lo:hi]
        sysl = slabs.SlabSystem(state, G, slabs.SlabComm("cpu"), theta=theta, group_dim=TG)
        gpu = slabs.PlanSlab(_params(case), device="cuda:0")
        for _ in range(STEPS):
            sysl.create_tree()
            sysl.summarize(gpu.bind(sysl).leaf_moments)
            sysl.evaluate(gpu)
            sysl.timestep(DT)
        acc = np.column_stack([sysl.state[:, 5], sysl.ax, sysl.ay])
        np.save(os.path.join(out_dir, f"rank{rank}.npy"), sysl.state)
        np.save(os.path.join(out_dir, f"acc{rank}.npy"), acc)
        gpu.close()
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("case", sorted(CASES))
def test_gpu_slab_step_equals_single_plan(tmp_path, case, oracle_mod):
    import torch.multiprocessing as mp

    from barneshut.gb300 import native

    ws = 2
    mp.start_processes(_worker, args=(ws, _free_port(), case, str(tmp_path)), nprocs=ws,
                       join=True, start_method="spawn")
    allp = np.concatenate([np.load(tmp_path / f"rank{r}.npy") for r in range(ws)])
    acc = np.concatenate([np.load(tmp_path / f"acc{r}.npy") for r in range(ws)])
    pid = allp[:, 5].astype(np.int64)
    assert np.array_equal(np.sort(pid), np.arange(N))
    got = allp[np.argsort(pid)]
    acc = acc[np.argsort(acc[:, 0])]

    # one plan over the whole system, the same phases and the same host tick
    theta, TG, eps, cut, dmin, qmin = CASES[case]
    x, y, m, vx, vy = _system()
    plan = native.Plan([N], [G], _params(case))
    for _ in range(STEPS):
        plan.load(x, y, m, vx, vy)
        plan.create_tree()
        plan.summarize()
        plan.evaluate()
        o = plan.store()  # particle-id order
        ax, ay = o["ax"].cpu().numpy(), o["ay"].cpu().numpy()
        if _ == STEPS - 1:
            ref_ax, ref_ay = ax, ay
            ox, oy = x, y  # positions the last accelerations were evaluated at
        vx, vy = vx + ax * DT, vy + ay * DT
        x, y = x + vx * DT, y + vy * DT
    assert oracle_mod.rel_rms(acc[:, 1], acc[:, 2], ref_ax, ref_ay) <= 1e-6
    assert np.max(np.abs(got[:, 0] - x)) <= 1e-9 and np.max(np.abs(got[:, 1] - y)) <= 1e-9
    # and against the FP64 oracle at the last step's positions
    oax, oay, _, _ = oracle_mod.theta_evaluate(ox, oy, m, G, TG=TG, theta=theta, eps2=eps * eps,
                                               cutoff=cut, dense_min=dmin, quad_min=max(qmin, 0))
    assert oracle_mod.rel_rms(acc[:, 1], acc[:, 2], oax, oay) <= 1e-5

#!/usr/bin/env python3
"""Throughput of the 2D grid-decomposition Barnes-Hut step on GB300.

Workload: N = 4,194,304 particles, seeded cluster mixture (8 Gaussians sigma
0.05 + 20 % uniform background, masses U[1,2), v = 0), 512 x 512 boxes, opening
angle 0.5, Plummer softening 1e-4, dt = 1e-5, G = 1, FP32 pair arithmetic with
Kahan-compensated far field.  The particle state (two FP64 buffers, ~400 MB)
is larger than L2, so no L2 flush is needed.

One "step" = one pass of the hot path over the same synthetic batch: reload
the seeded state from a device-resident copy (bh_load), then create_tree +
summarize + evaluate with the tick fused into the force epilogue (one
CUDA-graph replay).  The reload is inside the timed region.  It keeps every
timed step on the same distribution: with G = 1 and these masses the clusters
collapse within a few steps of dt = 1e-5, and a free-running simulation would
time a different (much denser) state at every step count.  The batch is
stored in the order the state has between steps of a running simulation (by
box, within a box by quadrant).

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
N > 1 runs under torchrun: every rank steps its own replica (weak scaling);
the path has no exchange step, so no collective is on the data path.

Prints one JSON line (rank 0).
"""
import argparse
import json
import os
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "barnes-hut_gb300"))
sys.path.insert(0, ROOT)

N_PART = 4_194_304
GRID = 512
THETA = 0.5
SOFTENING = 1e-4
DT = 1e-5
SEED = 2
METRIC = "particle-steps/s at N=4M on 1 GB300 (plain theta=0.5 step)"
WORKLOAD = "cluster-mixture N=4,194,304, 512x512 boxes, theta=0.5, eps=1e-4, dt=1e-5, FP32+Kahan"
K_FSTREAM_TRAFFIC = 1120.7e6  # bytes per force launch, dram read + write of one ncu capture


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--n", type=int, default=N_PART, help=argparse.SUPPRESS)
    ap.add_argument("--grid", type=int, default=GRID, help=argparse.SUPPRESS)
    ap.add_argument("--no-accuracy", action="store_true", help="skip the FP64 accuracy sample")
    ap.add_argument("--ref-sample-boxes", type=int, default=1024)
    ap.add_argument("--quick", action="store_true",
                    help="skip the autotuner and the batched / learned side measurements")
    ap.add_argument("--profile-learned", action="store_true",
                    help="for an ncu capture: train a small correction network, then run two "
                         "learned evaluates at N=1,048,576 (256 x 256 boxes, theta 0.8) and exit")
    ap.add_argument("--tile", default=None,
                    help="group_dim,dense_min,tune[,quad_min]: use this tile instead of the autotuner's")
    return ap.parse_args()


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def replica_seed(rank):
    """Seed of the batch a replica steps: every rank draws its own system."""
    return SEED + rank


def max_over_ranks(seconds, ws, device):
    """The slowest rank's time (the job finishes when it does); ws == 1 returns it as is.
    Works with any process-group backend whose all_reduce accepts tensors on `device`."""
    if ws <= 1:
        return float(seconds)
    import torch

    t = torch.tensor([float(seconds)], device=device, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in out.strip().splitlines():
            f = [v.strip() for v in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
                power.append(float(f[3]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm.sort()
        return {"sm_mhz": sm[len(sm) // 2], "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm), "power_w_max": max(power) if power else None}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def fp32_peak_tflops(torch, dev):
    """Measured FP32 SIMT peak: cuBLAS SGEMM 8192^3 with TF32 off (best of 5)."""
    prev = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    try:
        n = 8192
        a = torch.randn(n, n, device=dev)
        b = torch.randn(n, n, device=dev)
        c = torch.empty(n, n, device=dev)
        for _ in range(2):
            torch.matmul(a, b, out=c)
        best = 1e9
        for _ in range(5):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b, out=c)
            e1.record()
            e1.synchronize()
            best = min(best, e0.elapsed_time(e1) / 1e3)
        del a, b, c
        return 2.0 * n ** 3 / best / 1e12
    finally:
        torch.backends.cuda.matmul.allow_tf32 = prev


def cpu_baseline(x, y, m, G, full_limit_s=240.0):
    """The reference CPU algorithm -- the oracle's restatement of sequential.py and
    com_concat_dedup (evaluation.py:73-109), FP64, OpenMP over target boxes on every host core --
    on the bench's own input.  First a bounded sample: the O(N) phases (bounding box, keys, the
    structured sort, COMs) in full and the evaluation of 1,024 non-empty boxes at a fixed stride,
    scaled to all boxes to estimate a step.  Then, when that estimate is within full_limit_s, one
    full step (every non-empty box evaluated), whose measured time is the reported baseline."""
    from oracle import oracle

    threads = os.cpu_count() or 1
    est = oracle.reference_sample_time(x, y, m, G, 1024, threads)
    out = {"unit": "particle-steps/s", "cores": threads, "kind": "port",
           "estimate_s": est["step_s"], "estimate_sample": f"{est['sampled']} of {est['nonempty']} boxes"}
    if est["step_s"] <= full_limit_s:
        full = oracle.reference_sample_time(x, y, m, G, 1 << 40, threads)
        step_s = full["setup_s"] + full["sample_s"]
        out.update(value=len(x) / step_s, step_seconds=step_s, measured="full step",
                   sample=(f"one full reference CPU step measured on the same N={len(x)} input: O(N) "
                           f"phases {full['setup_s']:.2f} s + evaluation of all {full['nonempty']} "
                           f"non-empty boxes {full['sample_s']:.1f} s (the sampled estimate, "
                           f"{est['sampled']} boxes scaled up, was {est['step_s']:.1f} s)"))
    else:
        out.update(value=len(x) / est["step_s"], step_seconds=est["step_s"], measured="estimate",
                   sample=(f"reference CPU step estimated on the same N={len(x)} input: O(N) phases "
                           f"in full ({est['setup_s']:.2f} s) + evaluation of {est['sampled']} of "
                           f"{est['nonempty']} non-empty boxes ({est['sample_s']:.2f} s), scaled to "
                           f"{est['step_s']:.1f} s/step (a full step exceeds {full_limit_s:.0f} s)"))
    return out


def cpu_estimator_check(n=1 << 20, G=256, seed=1):
    """The sampled estimate of a reference CPU step against a full measured step at N = 1,048,576
    on 256 x 256 boxes (a few seconds on the host): how far the scaled sample is from the truth."""
    from barneshut.gb300 import workloads
    from oracle import oracle

    x, y, m, _, _ = workloads.cluster_mixture(n, seed=seed)
    threads = os.cpu_count() or 1
    est = oracle.reference_sample_time(x, y, m, G, 1024, threads)
    full = oracle.reference_sample_time(x, y, m, G, 1 << 40, threads)
    full_s = full["setup_s"] + full["sample_s"]
    return {"n": n, "grid": G, "cores": threads, "full_step_s": full_s, "estimated_step_s": est["step_s"],
            "estimate_over_full": est["step_s"] / full_s}


def flat_same_config(torch, dev, batch, host, reps=2):
    """The reference's own algorithm on the GPU at the bench's N = 4,194,304 / 512 x 512 input:
    flat far field (every non-neighbour box through its centre of mass), 3 x 3 near field, the
    CPU path's r^2 <= 1e-5 cutoff, no softening, FP32 pairs with Kahan far field.  Step time
    (create_tree + summarize + evaluate + tick, CUDA events) and relative RMS force error on
    16,384 seeded targets against the FP64 restatement of the reference evaluation."""
    from barneshut.gb300 import native, workloads
    from oracle import oracle

    n = batch[0].numel()
    prm = native.make_params(1.0, DT, 0.0, 1e-5, 0.0, 0, native.BH_PREC_FP32_KAHAN)
    plan = native.Plan([n], [GRID], prm, device=dev)
    stream = torch.cuda.current_stream(dev)
    plan.load(*batch)
    plan.step(1)  # warm-up
    ms = []
    for _ in range(reps):
        plan.load(*batch)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.step(1)
        e1.record(stream)
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    plan.load(*batch)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    o = plan.store()
    near, far = plan.pair_counts()
    flags = plan.error_flags(raise_on_error=False)
    plan.close()
    t = workloads.precision_subsample(n, 16384, seed=SEED)
    x, y, m = host
    rax, ray = oracle.gpu_evaluate(x, y, m, GRID, gconst=1.0, cutoff=1e-5, targets=t)
    ax, ay = o["ax"].cpu().numpy()[t], o["ay"].cpu().numpy()[t]
    ms_step = sorted(ms)[len(ms) // 2]
    return {"workload": "reference algorithm: flat far field, r^2 <= 1e-5 cutoff, no softening, "
                        "FP32+Kahan pairs",
            "ms_per_step": ms_step, "particle_steps_per_s": n / (ms_step / 1e3),
            "rel_rms_vs_reference_cpu_algorithm": oracle.rel_rms(ax, ay, rax[t], ray[t]),
            "targets": len(t), "pairs_near": near, "pairs_far": far, "device_error_flags": flags}


def batched_benchmark(torch, dev, nsys=512, steps=50, warmup=3):
    """512 independent systems (log-uniform N in [1024, 262144], uniform or 4-cluster,
    ~64 particles per box, theta 0.5, FP32) stepped together: every phase is one launch
    over all systems (the force kernel a persistent work queue), the step one CUDA graph."""
    import numpy as np

    from barneshut.gb300 import autotune, native, workloads

    systems, grids = workloads.batched_systems(nsys, seed=4)
    n = [len(s[0]) for s in systems]
    tile, _ = autotune.tune(systems, grids, 1.0, 1e-6, 1e-4, 0.5, device=dev)
    prm = native.make_params(1.0, 1e-6, 1e-4, 0.0, 0.5, tile["group_dim"],
                             native.BH_PREC_FP32_KAHAN, 0, tile["tune"], dense_min=tile.get("dense_min", 0),
                             quad_min=tile.get("quad_min", 0))
    plan = native.Plan(n, grids, prm, device=dev)
    plan.load(*[np.concatenate([s[k] for s in systems]) for k in range(5)])
    for _ in range(warmup):
        plan.step_graph(1)
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plan.step_graph(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    # one more step's force kernel alone (CUDA events around it) with its pair counts: the
    # batched line's FP32 roofline (12 flop per near pair, 20 per far pair)
    plan.set_kernel_timing(True)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    kms = plan.force_kernel_ms()
    nn, nf = plan.pair_counts()
    flags = plan.error_flags(raise_on_error=False)
    out = {"metric": "particle-steps/s, 512 batched systems", "value": sum(n) * steps / t,
           "systems": nsys, "particles": int(sum(n)), "steps": steps, "ms_per_step": 1e3 * t / steps,
           "theta": 0.5, "dt": 1e-6, "tile": tile, "graph": f"{steps} steps in one CUDA graph",
           "kernels_per_step": plan.kernels_per_step(),
           "force_kernel": {"ms": kms, "pairs_near": nn, "pairs_far": nf,
                            "tflops": (12.0 * nn + 20.0 * nf) / kms / 1e9},
           "device_error_flags": flags}
    plan.close()
    return out


def _rel_rms_t(torch, ax, ay, dax, day):
    return float(torch.sqrt(((ax - dax) ** 2 + (ay - day) ** 2).sum() / (dax ** 2 + day ** 2).sum()))


def learned_benchmark(torch, dev, batch, steps=20, n_pairs=10_000_000,
                      plain_thetas=(0.4, 0.45, 0.5, 0.55, 0.6, 0.65, 0.7, 0.8),
                      learned_thetas=(0.55, 0.6, 0.65, 0.7, 0.8)):
    """Learned far-field correction: the network is trained on n_pairs (target, cell) pairs the
    method generates on two seeded cluster-mixture systems (N = 1,048,576, 256 x 256 boxes; cells
    accepted at theta 0.8 but opened at 0.5), then applied on the bench's N = 4,194,304 batch at
    several opening angles (correction_theta 0.5: the cells accepted at theta but opened at 0.5
    are corrected).  For every plain and learned opening angle: step time (CUDA events over
    `steps` graph replays, the reload included as in the headline) and relative RMS force error
    against the FP64 direct sum on the same 16,384 targets -- the two Pareto curves."""
    import time as _t

    from barneshut.gb300 import learned, native, workloads

    t0 = _t.time()
    train = [workloads.cluster_mixture(1 << 20, seed=11), workloads.cluster_mixture(1 << 20, seed=12)]
    mlp, info = learned.train_correction(train, 256, 0.8, 0.5, n_pairs=n_pairs, epochs=4)
    train_s = _t.time() - t0
    n = batch[0].numel()
    tgt = workloads.precision_subsample(n, 16384, seed=SEED)
    idx = torch.as_tensor(tgt, device=dev)
    stream = torch.cuda.current_stream(dev)
    ref = None
    rows = []
    for kind, thetas in (("plain", plain_thetas), ("learned", learned_thetas)):
        for theta in thetas:
            flags = native.BH_FLAG_LEARNED if kind == "learned" else 0
            prm = native.make_params(1.0, DT, SOFTENING, 0.0, theta, 0, native.BH_PREC_FP32_KAHAN,
                                     flags, 0, 0.5)
            plan = native.Plan([n], [GRID], prm, device=dev)
            if flags:
                plan.set_correction(mlp)
            for _ in range(3):
                plan.load(*batch)
                plan.step_graph(1)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                plan.load(*batch)
                plan.step_graph(1)
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / steps
            plan.load(*batch)
            plan.create_tree()
            plan.summarize()
            plan.evaluate()
            o = plan.store()
            if ref is None:
                ref = plan.direct_sample(tgt)
            err = _rel_rms_t(torch, o["ax"][idx], o["ay"][idx], *ref)
            near, far = plan.pair_counts()
            rows.append({"kind": kind, "theta": theta, "ms_per_step": ms,
                         "particle_steps_per_s": n / (ms / 1e3), "rel_rms_vs_fp64_direct": err,
                         "pairs_near": near, "pairs_far": far,
                         "pairs_corrected": plan.corrected_pairs() if flags else 0,
                         "device_error_flags": plan.error_flags(raise_on_error=False)})
            plan.close()
    plain = [r for r in rows if r["kind"] == "plain"]
    best = {}
    for r in rows:
        if r["kind"] != "learned":
            continue
        # the fastest plain step at least as accurate as this learned step
        ok = [p for p in plain if p["rel_rms_vs_fp64_direct"] <= r["rel_rms_vs_fp64_direct"]]
        fastest = min(ok, key=lambda p: p["ms_per_step"]) if ok else None
        best[f"learned_{r['theta']}"] = {
            "matched_plain_theta": fastest["theta"] if fastest else None,
            "learned_over_plain_time": r["ms_per_step"] / fastest["ms_per_step"] if fastest else None}
    return {"pareto": rows, "matched_error": best,
            "training": {"pairs": info["pairs"], "relative_mse": info["relative_mse"],
                         "quadrupole_only_relative_mse": info["quadrupole_relative_mse"],
                         "loss_history": info["loss_history"], "seconds": train_s}}


def precision_study(torch, dev, batch, thetas=(0.3, 0.5, 0.7), reps=3):
    """Force error of FP32 naive, FP32 with Kahan far field and FP64 pair arithmetic against the
    FP64 direct sum on 16,384 seeded targets of the bench's N = 4,194,304 batch (512 x 512 boxes),
    at each opening angle.  The three arithmetic columns run the same force path (the pyramid
    walk, BH_FLAG_WALK, whose interaction lists do not depend on the arithmetic), so they differ
    in arithmetic alone: equal pair counts, and the FP32 columns' difference from the FP64 column
    is reported beside their error.  A fourth column is the production path (list streaming with
    refined lists, FP32 + Kahan), with its own lists.  Evaluate time: median of `reps` launches."""
    from barneshut.gb300 import native, workloads

    n = batch[0].numel()
    tgt = workloads.precision_subsample(n, 16384, seed=SEED)
    idx = torch.as_tensor(tgt, device=dev)
    stream = torch.cuda.current_stream(dev)
    ref = None
    out = {"targets": len(tgt), "n": n, "grid": GRID}
    cols = (("fp32", native.BH_PREC_FP32, native.BH_FLAG_WALK),
            ("fp32_kahan", native.BH_PREC_FP32_KAHAN, native.BH_FLAG_WALK),
            ("fp64", native.BH_PREC_FP64, native.BH_FLAG_WALK),
            ("fp32_kahan_stream", native.BH_PREC_FP32_KAHAN, 0))
    for theta in thetas:
        row, acc = {}, {}
        for name, prec, flags in cols:
            prm = native.make_params(1.0, DT, SOFTENING, 0.0, theta, 0, prec, flags, 0)
            plan = native.Plan([n], [GRID], prm, device=dev)
            plan.load(*batch)
            plan.create_tree()
            plan.summarize()
            ms = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                plan.evaluate()
                e1.record(stream)
                torch.cuda.synchronize()
                ms.append(e0.elapsed_time(e1))
            # evaluate accumulates into a: one clean pass for the error and the pair counts
            plan.load(*batch)
            plan.create_tree()
            plan.summarize()
            plan.evaluate()
            o = plan.store()
            if ref is None:
                ref = plan.direct_sample(tgt)
            dax, day = ref
            ax, ay = o["ax"][idx], o["ay"][idx]
            acc[name] = (ax, ay)
            mag = torch.sqrt(dax ** 2 + day ** 2)
            rel = torch.sqrt((ax - dax) ** 2 + (ay - day) ** 2) / mag
            near, far = plan.pair_counts()
            row[name] = {"rel_rms": _rel_rms_t(torch, ax, ay, dax, day),
                         "rel_max": float(rel.max()), "evaluate_ms": sorted(ms)[len(ms) // 2],
                         "pairs_near": near, "pairs_far": far,
                         "device_error_flags": plan.error_flags(raise_on_error=False)}
            plan.close()
        for name in ("fp32", "fp32_kahan"):
            row[name]["rel_rms_vs_fp64_column"] = _rel_rms_t(torch, *acc[name], *acc["fp64"])
        out[f"theta_{theta}"] = row
    return out


def free_run(torch, dev, steps=100):
    """N = 1,048,576 cluster mixture (seed 1), 256 x 256 boxes, theta 0.5, softening 1e-4,
    dt 1e-5, FP32 + Kahan: `steps` free-running steps in one CUDA graph, with FP64 kinetic
    energy and momentum before and after (the ln-potential diagnostic is O(N^2) and is left
    out at this size)."""
    import numpy as np

    from barneshut.gb300 import native, workloads

    x, y, m, vx, vy = workloads.cluster_mixture(1 << 20, seed=1)
    n = len(x)
    prm = native.make_params(1.0, 1e-5, 1e-4, 0.0, 0.5, 0, native.BH_PREC_FP32_KAHAN, 0, 0)
    plan = native.Plan([n], [256], prm, device=dev)
    plan.load(x, y, m, vx, vy)
    plan.step_graph(3)  # graph capture and warm-up
    plan.load(x, y, m, vx, vy)
    torch.cuda.synchronize()
    ke0, px0, py0, _ = plan.diagnostics()
    stream = torch.cuda.current_stream(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    plan.step_graph(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3
    ke1, px1, py1, _ = plan.diagnostics()
    o = plan.store()
    msum = float(np.sum(m))
    speed = torch.sqrt(o["vx"] ** 2 + o["vy"] ** 2)
    mv = float((torch.as_tensor(m, device=dev) * speed).sum())
    res = {"metric": "particle-steps/s, N=1M free-running", "value": n * steps / t,
           "ms_per_step": 1e3 * t / steps, "steps": steps, "n": n, "grid": 256,
           "graph": f"{steps} steps in one CUDA graph",
           "kinetic_energy": [ke0, ke1],
           "momentum_drift_over_sum_m_abs_v": float(np.hypot(px1 - px0, py1 - py0) / mv) if mv > 0 else None,
           "total_mass": msum,
           "device_error_flags": plan.error_flags(raise_on_error=False)}
    plan.close()
    return res


def e2e_serial_ms(torch, plan, host_in, dev, stream, steps):
    """ms per step of H2D inputs -> bh_load -> bh_step_graph(1) -> bh_store -> D2H results, one
    stream, nothing overlapped."""
    n = host_in[0].numel()
    dev_in = [torch.empty_like(h, device=dev) for h in host_in]
    host_out = [torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(6)]

    def one():
        for h, d in zip(host_in, dev_in):
            d.copy_(h, non_blocking=True)
        plan.load(*dev_in)
        plan.step_graph(1)
        outs = plan.store()
        for h, k in zip(host_out, ("x", "y", "vx", "vy", "ax", "ay")):
            h.copy_(outs[k], non_blocking=True)

    for _ in range(2):
        one()
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(stream)
    for _ in range(steps):
        one()
    g1.record(stream)
    torch.cuda.synchronize()
    return g0.elapsed_time(g1) / steps


def e2e_pipelined_ms(torch, plan, host_in, dev, steps):
    """ms per step of the same sequence with three streams: H2D of step k's inputs into device
    buffer k % 2 (after step k - 2's bh_load has read it), the step on the compute stream
    (bh_load, bh_step_graph(1), bh_store into device buffer k % 2 once step k - 2's results have
    left it), and D2H of step k's results into pinned host buffer k % 2.  Every step's inputs
    and results cross the host link inside the timed region."""
    import ctypes

    from barneshut.gb300 import native

    n = host_in[0].numel()
    s_h2d, s_cmp, s_d2h = (torch.cuda.Stream(dev) for _ in range(3))
    dev_in = [[torch.empty_like(h, device=dev) for h in host_in] for _ in range(2)]
    dev_out = [[torch.empty(n, dtype=torch.float64, device=dev) for _ in range(6)] for _ in range(2)]
    host_out = [[torch.empty(n, dtype=torch.float64).pin_memory() for _ in range(6)] for _ in range(2)]
    ev = {k: [torch.cuda.Event() for _ in range(2)] for k in ("h2d", "loaded", "stored", "d2h")}
    L = native.load_library()

    def issue(k):
        b = k % 2
        with torch.cuda.stream(s_h2d):
            if k >= 2:
                s_h2d.wait_event(ev["loaded"][b])
            for h, d in zip(host_in, dev_in[b]):
                d.copy_(h, non_blocking=True)
            ev["h2d"][b].record(s_h2d)
        with torch.cuda.stream(s_cmp):
            s_cmp.wait_event(ev["h2d"][b])
            st = ctypes.c_void_p(s_cmp.cuda_stream)
            plan._check(L.bh_load(plan.h, *[native._ptr(t) for t in dev_in[b]], st))
            ev["loaded"][b].record(s_cmp)
            plan._check(L.bh_step_graph(plan.h, 1, st))
            if k >= 2:
                s_cmp.wait_event(ev["d2h"][b])
            plan._check(L.bh_store(plan.h, *[native._ptr(t) for t in dev_out[b]], st))
            ev["stored"][b].record(s_cmp)
        with torch.cuda.stream(s_d2h):
            s_d2h.wait_event(ev["stored"][b])
            for h, d in zip(host_out[b], dev_out[b]):
                h.copy_(d, non_blocking=True)
            ev["d2h"][b].record(s_d2h)

    for k in range(3):  # warm-up (graph already captured on the plan)
        issue(k)
    torch.cuda.synchronize()
    g0, g1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g0.record(s_h2d)
    s_cmp.wait_event(g0)
    s_d2h.wait_event(g0)
    for k in range(steps):
        issue(k)
    g1.record(s_d2h)  # after the last D2H, which follows every step's work
    torch.cuda.synchronize()
    return g0.elapsed_time(g1) / steps


def run_reference(args, ws, rank):
    """The reference arm: the reference's CPU algorithm (the oracle's restatement of
    sequential.py + com_concat_dedup, FP64, OpenMP over target boxes on every host core) on the
    same N = 4,194,304 / 512 x 512 input.  A full step takes minutes on the host, so each of the
    W + K steps is a bounded sample of one: the O(N) phases (bounding box, keys, the structured
    sort, COMs) in full and the evaluation of `--ref-sample-boxes` non-empty boxes at a fixed
    stride, step k starting one box further along the stride (the K timed steps evaluate K
    disjoint box samples).  ms_per_step is the measured time of those sampled steps; value is
    N / (O(N) time + evaluation time scaled to all non-empty boxes), averaged over the K steps.
    Under torchrun only rank 0 runs."""
    if rank != 0:
        return
    from barneshut.gb300 import workloads
    from oracle import oracle

    x, y, m, vx, vy = workloads.cluster_mixture(args.n, seed=SEED)
    threads = os.cpu_count() or 1
    K, W = max(1, args.steps), max(0, args.warmup)
    for k in range(W):
        oracle.reference_sample_time(x, y, m, args.grid, args.ref_sample_boxes, threads, offset=k)
    t0 = time.perf_counter()
    runs = [oracle.reference_sample_time(x, y, m, args.grid, args.ref_sample_boxes, threads,
                                         offset=W + k) for k in range(K)]
    timed = time.perf_counter() - t0
    est_s = sum(r["step_s"] for r in runs) / K
    val = args.n / est_s
    r0 = runs[0]
    sample = (f"each step: O(N) phases in full (mean {sum(r['setup_s'] for r in runs) / K:.2f} s) + "
              f"evaluation of {r0['sampled']} of {r0['nonempty']} non-empty boxes (mean "
              f"{sum(r['sample_s'] for r in runs) / K:.2f} s), K disjoint box samples; value = N / "
              f"(O(N) time + evaluation time x {r0['nonempty']}/{r0['sampled']}) = N / {est_s:.1f} s")
    line = {"metric": METRIC, "value": val, "unit": "particle-steps/s", "n_gpus": args.gpus,
            "steps": K, "warmup": W, "ms_per_step": 1e3 * timed / K,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "impl": "reference",
            "config": {"workload": WORKLOAD + " (reference algorithm: flat far field, r^2 <= 1e-5 "
                                              "cutoff; the reference has no opening angle)",
                       "n": args.n, "grid": args.grid},
            "cpu_baseline": {"value": val, "unit": "particle-steps/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": val, "unit": "particle-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "estimated_full_step_s": est_s}
    print(json.dumps(line), flush=True)


def profile_learned():
    """Two learned evaluates at N = 1,048,576 (cluster mixture seed 1, 256 x 256 boxes, theta 0.8,
    correction theta 0.5) with a network trained on 2^19 pairs of a 2^18-particle system: a small
    case for capturing k_learned_correct under ncu (the second launch)."""
    import torch

    from barneshut.gb300 import learned, native, workloads

    mlp, _ = learned.train_correction([workloads.cluster_mixture(1 << 18, seed=11)], 128, 0.8, 0.5,
                                      n_pairs=1 << 19, epochs=1)
    x, y, m, vx, vy = workloads.cluster_mixture(1 << 20, seed=1)
    prm = native.make_params(1.0, DT, SOFTENING, 0.0, 0.8, 0, native.BH_PREC_FP32_KAHAN,
                             native.BH_FLAG_LEARNED, 0, 0.5)
    plan = native.Plan([len(x)], [256], prm)
    plan.set_correction(mlp)
    ms = []
    for _ in range(2):
        plan.load(x, y, m, vx, vy)
        plan.create_tree()
        plan.summarize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        plan.evaluate()
        e1.record()
        torch.cuda.synchronize()
        ms.append(e0.elapsed_time(e1))
    near, far = plan.pair_counts()
    print(json.dumps({"profile": "learned", "n": len(x), "grid": 256, "theta": 0.8,
                      "evaluate_ms": ms, "pairs_corrected": plan.corrected_pairs(),
                      "pairs_near": near, "pairs_far": far,
                      "device_error_flags": plan.error_flags(raise_on_error=False)}), flush=True)


def main():
    args = parse()
    ws, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, ws, rank)
        return
    if args.profile_learned:
        profile_learned()
        return
    import numpy as np
    import torch

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=dev)
    from barneshut.gb300 import native, workloads

    x, y, m, vx, vy = workloads.cluster_mixture(args.n, seed=replica_seed(rank))
    # batch in the state's order between steps of a running simulation (box, then quadrant)
    order = workloads.box_order(x, y, args.grid)
    x, y, m, vx, vy = (a[order].copy() for a in (x, y, m, vx, vy))
    tile = {"group_dim": 0, "tune": 0, "dense_min": 0}
    tune_ms = None
    if args.tile:
        v = [int(t) for t in args.tile.split(",")]
        tile = {"group_dim": v[0], "dense_min": v[1], "tune": v[2], "quad_min": v[3] if len(v) > 3 else 0}
    elif not args.quick:
        from barneshut.gb300 import autotune

        tile, tt = autotune.tune([(x, y, m, vx, vy)], [args.grid], 1.0, DT, SOFTENING, THETA,
                                 device=dev)
        tune_ms = {k: round(1e3 * v, 3) for k, v in tt.items()}
    prm = native.make_params(1.0, DT, SOFTENING, 0.0, THETA, tile["group_dim"],
                             native.BH_PREC_FP32_KAHAN, 0, tile["tune"], dense_min=tile.get("dense_min", 0),
                             quad_min=tile.get("quad_min", 0))
    plan = native.Plan([args.n], [args.grid], prm, device=dev)
    stream = torch.cuda.current_stream(dev)
    batch = [torch.from_numpy(a).to(dev) for a in (x, y, m, vx, vy)]

    def one_step():
        plan.load(*batch)
        plan.step_graph(1)

    # ---- warmup (graph capture happens on the first replay)
    W = max(3, args.warmup)
    for _ in range(W):
        one_step()
    torch.cuda.synchronize()
    plan.error_flags()

    # ---- timed region: K graph replays, inputs resident in HBM
    K = args.steps
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(K):
        one_step()
    e1.record(stream)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    clk = clocks.stop()
    t_dev = max_over_ranks(e0.elapsed_time(e1) / 1e3, ws, dev)
    value = ws * args.n * K / t_dev
    flags = plan.error_flags(raise_on_error=False)
    kernels_per_step = plan.kernels_per_step()

    # ---- phases (CUDA events): load, create_tree, summarize, force (dominant kernel)
    ph = {"load": [], "create_tree": [], "summarize": [], "force": []}
    kern = []
    plan.set_kernel_timing(True)
    for _ in range(max(3, min(K, 10))):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        ev[0].record(stream)
        plan.load(*batch)
        ev[1].record(stream)
        plan.create_tree()
        ev[2].record(stream)
        plan.summarize()
        ev[3].record(stream)
        plan.evaluate()
        ev[4].record(stream)
        torch.cuda.synchronize()
        for k, (a, b) in zip(ph, zip(ev[:-1], ev[1:])):
            ph[k].append(a.elapsed_time(b))
        kern.append(plan.force_kernel_ms())
    plan.set_kernel_timing(False)
    phases_ms = {k: sorted(v)[len(v) // 2] for k, v in ph.items()}
    near2, far2 = plan.pair_counts()
    t_kernel = sum(kern) / len(kern) / 1e3  # the force kernel alone, mean over the launches
    flops_force = 12.0 * near2 + 20.0 * far2
    peak = fp32_peak_tflops(torch, dev)

    # ---- e2e through the C ABI with host buffers: every step copies its inputs from pinned host
    # memory, steps, and copies its results back.  Measured twice: serially on one stream, and
    # pipelined (the copy of step k + 1's inputs and of step k - 1's results overlap step k).
    host_in = [torch.from_numpy(np.ascontiguousarray(a)).pin_memory() for a in (x, y, m, vx, vy)]
    e2e_serial = e2e_serial_ms(torch, plan, host_in, dev, stream, max(3, min(K, 10)))
    e2e_steps = max(6, K)  # the timed step count of `value`: steady state, as there
    t_e2e = e2e_pipelined_ms(torch, plan, host_in, dev, e2e_steps) / 1e3
    if ws > 1:
        torch.distributed.barrier()
    t_e2e = max_over_ranks(t_e2e, ws, dev)
    e2e = {"value": ws * args.n / t_e2e, "unit": "particle-steps/s",
           "h2d_bytes_per_step": ws * 5 * 8 * args.n, "d2h_bytes_per_step": ws * 6 * 8 * args.n,
           "ms_per_step": 1e3 * t_e2e, "steps": e2e_steps,
           "path": ("pinned host arrays -> bh_load -> bh_step_graph(1) -> bh_store -> pinned host, "
                    "every step; three streams and double-buffered device arrays let the copies of "
                    "step k + 1's inputs and step k - 1's results overlap step k (the first copy in "
                    "and the last copy out are not overlapped)"),
           "serial_ms_per_step": e2e_serial}

    # ---- accuracy of the measured step vs FP64 direct sum (on the device)
    acc = None
    if not args.no_accuracy:
        plan.load(*batch)
        plan.create_tree()
        plan.summarize()
        plan.evaluate()
        o = plan.store()
        t = workloads.precision_subsample(args.n, 16384, seed=SEED)
        dax, day = plan.direct_sample(t)
        ax, ay = o["ax"][torch.as_tensor(t, device=dev)], o["ay"][torch.as_tensor(t, device=dev)]
        num = ((ax - dax) ** 2 + (ay - day) ** 2).sum()
        den = (dax ** 2 + day ** 2).sum()
        mag = torch.sqrt(dax ** 2 + day ** 2)
        rel = torch.sqrt((ax - dax) ** 2 + (ay - day) ** 2) / mag
        acc = {"rel_rms_vs_fp64_direct": float(torch.sqrt(num / den)),
               "rel_max_vs_fp64_direct": float(rel.max()), "targets": int(len(t))}

    side = {}
    if not args.quick and rank == 0:
        side["batched"] = batched_benchmark(torch, dev)
        fk = side["batched"]["force_kernel"]
        fk["frac_of_sgemm"] = fk["tflops"] / peak if peak else None
        side["free_run_1m"] = free_run(torch, dev)
        side["precision"] = precision_study(torch, dev, batch)
        side["learned"] = learned_benchmark(torch, dev, batch)

    if not args.quick and rank == 0:
        side["flat_same_config"] = flat_same_config(torch, dev, batch, (x, y, m))
        side["cpu_estimator_check"] = cpu_estimator_check()
    cpu = None
    if rank == 0:
        cpu = cpu_baseline(x, y, m, args.grid, full_limit_s=0.0 if args.quick else 240.0)

    if rank == 0:
        peaks = measured_peaks()
        achieved = flops_force / t_kernel / 1e12
        nominal = 152 * 128 * 2 * (clk.get("sm_max_mhz") or 2070.0) * 1e6 / 1e12
        line = {
            "metric": METRIC, "value": value, "unit": "particle-steps/s", "n_gpus": ws,
            "steps": K, "warmup": W, "ms_per_step": 1e3 * t_dev / K, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "n": args.n, "grid": args.grid, "theta": THETA,
                       "softening": SOFTENING, "dt": DT, "seed": SEED,
                       "l2": "state ~400 MB > 129 MB L2 (no flush needed)",
                       "parallelism": f"{ws} independent replica(s)"},
            "gpu_launches": (kernels_per_step + 1) * K,  # + the bh_load kernel of each step
            "roofline": {"bound": "fp32", "kernel": "k_fstream (list-streaming force kernel, tick fused)",
                         "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                         "frac": achieved / peak, "traffic": K_FSTREAM_TRAFFIC,
                         "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one "
                                           "k_fstream launch at this workload (committed summary)",
                         "peak_source": "measured in this run: cuBLAS SGEMM 8192^3, TF32 off "
                                        "(MEASURED_PEAKS.json has no FP32 figure)",
                         "nominal_peak": nominal, "frac_of_nominal": achieved / nominal,
                         "algorithmic": f"12 flop x {near2} near + 20 flop x {far2} far pairs",
                         "kernel_ms": 1e3 * t_kernel,
                         "kernel_ms_source": "CUDA events around the force kernel alone "
                                             "(bh_set_kernel_timing), mean of the phase launches",
                         "force_phase_ms": phases_ms["force"]},
            "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
            "cpu_baseline_detail": {k: cpu[k] for k in ("measured", "step_seconds", "estimate_s",
                                                       "estimate_sample")},
            "e2e": e2e,
            "clocks": clk,
            "accuracy": acc,
            "pairs_per_step": {"near": near2, "far": far2},
            "phases_ms": phases_ms,
            "tile": {"chosen": tile, "autotune_force_ms": tune_ms},
            **side,
            "device_error_flags": flags,
            "reference_recorded": {"value": 10_000_000 / 166.837, "unit": "particle-steps/s",
                                   "note": "python-bh singlegpu, N=10M, flat far field, FP64, "
                                           "unstated GPU (data/frontera/nbody_out_singlegpu.dat)"},
            "measured_peaks": {k: peaks.get(k) for k in ("hbm_gbs", "bf16_tflops")},
        }
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()

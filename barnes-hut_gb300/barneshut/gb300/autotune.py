"""Autotuner for the force kernel's tile shape.

Tunables (per plan): group_dim -- target group edge in leaf boxes (1, 2, 4 or 8;
TG^2 boxes share one interaction list) --, dense_min -- boxes holding at least
this many particles get their own work items and per-box refined near lists
(list-streaming path) --, quad_min -- boxes holding at least this many particles
are refined quadrant by quadrant (-1: never) -- and tune -- the list-streaming kernel's build
(0: 6 CTAs per SM with 80 registers per thread, 1: 8 CTAs per SM with 64).  Every candidate keeps
the opening-angle rule for every target (a cell accepted for a group rectangle
passes the test for each of its boxes); they differ in how far the lists are
refined, so the chosen one's accuracy is measured and reported by the caller.
Candidates are timed with CUDA events on the caller's own particles
(create_tree + summarize once, then the force phase alone, median of a few
launches); the fastest is returned and cached in memory (and optionally in a
JSON file) under a key made of the workload's shape: particle count, grid,
opening angle, softening and occupancy per box.
"""
import json
import math
import os

from . import native

_CACHE = {}


def _key(n, grids, theta, softening, precision):
    nb = sum(n) / max(1, sum(g * g for g in grids))
    return json.dumps({"n": int(2 ** round(math.log2(max(1, sum(n))))), "nsys": len(n),
                       "G": int(2 ** round(math.log2(max(1, max(grids))))),
                       "theta": round(float(theta), 3), "eps": float(softening),
                       "per_box": round(math.log2(max(nb, 1e-3))), "prec": int(precision)},
                      sort_keys=True)


def candidates(theta):
    out = []
    for tg in (1, 2, 4, 8):
        for dm in ((0,) if tg == 1 else (16, 32, 64)):
            for qm in (-1, 128):
                for tune in (0, 1):
                    out.append({"group_dim": tg, "dense_min": dm, "quad_min": qm, "tune": tune})
    return out


def tune(systems, grids, grav_constant=1.0, dt=1e-5, softening=1e-4, theta=0.5,
         precision=native.BH_PREC_FP32_KAHAN, repeats=3, device="cuda", cache_path=None,
         log=None):
    """Pick {group_dim, dense_min, tune} for these systems (list of (x, y, m, vx, vy)).

    Returns (best config dict, {config: seconds} timings)."""
    import numpy as np
    import torch

    n = [len(s[0]) for s in systems]
    key = _key(n, grids, theta, softening, precision)
    if cache_path and os.path.exists(cache_path) and not _CACHE:
        with open(cache_path) as f:
            _CACHE.update(json.load(f))
    if key in _CACHE:
        return _CACHE[key]["best"], _CACHE[key]["timings"]
    cat = [np.concatenate([s[k] for s in systems]) for k in range(5)]
    timings = {}
    stream = torch.cuda.current_stream(device)
    for c in candidates(theta):
        prm = native.make_params(grav_constant, dt, softening, 0.0, theta, c["group_dim"],
                                 precision, 0, c["tune"], dense_min=c["dense_min"],
                                 quad_min=c["quad_min"])
        try:
            plan = native.Plan(n, grids, prm, device=device)
        except native.BHError:
            continue
        plan.load(*cat)
        plan.create_tree()
        plan.summarize()
        plan.evaluate()  # warm-up
        ts = []
        for _ in range(repeats):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            plan.evaluate()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        plan.error_flags()
        timings[json.dumps(c, sort_keys=True)] = sorted(ts)[len(ts) // 2]
        if log:
            log(f"autotune {c}: {1e3 * timings[json.dumps(c, sort_keys=True)]:.3f} ms")
        plan.close()
        del plan
    best = json.loads(min(timings, key=timings.get))
    _CACHE[key] = {"best": best, "timings": timings}
    if cache_path:
        with open(cache_path, "w") as f:
            json.dump(_CACHE, f, indent=1, sort_keys=True)
    return best, timings

#!/usr/bin/env python3
"""Generate golden vectors by running the reference python-bh CPU path.

The reference (ut-parla/barnes-hut, ``python-bh``) ships no tests and no
result vectors, so its own CPU implementation is the thing that pins parity.
This script imports ``barneshut.implementations.sequential.SequentialBarnesHut``
from a checkout of the reference and drives its step phases exactly as
``implementations/base.py:94-135`` does (``create_tree`` -> ``summarize`` ->
``evaluate``), with two documented deviations that make a multi-step run
meaningful:

* the reference CPU ``timestep`` is a no-op (``grid_decomposition/box.py:26-30``
  tests the bound method ``self.cloud.is_empty``, which is always truthy), so
  the tick of the reference GPU path, ``kernels/grid_decomposition/gpu/grid.py:159-174``
  (v += a*dt; a = 0; x += v*dt), is applied here to the particle array;
* ``numba`` is not installed, so a stub (``numba_stub/``) turns ``@njit`` into
  an identity decorator; the same source then runs as float64 NumPy code.

Usage (needs a reference checkout; run once, commit the ``.npz`` output):

    python tests/golden/make_golden.py /path/to/reference/python-bh

Outputs ``tests/golden/ref_<case>.npz``.  Each file holds the inputs, the
config, and per recorded step the particle box keys, the box centres of mass
and the accelerations in original particle (pid) order, plus the state after
the last step.
"""
import contextlib
import io
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

INI_TEMPLATE = """[general]
implementation = sequential
sample_check_size = 10
skip_timestep = False
evaluation_rounds = 1
rounds = 1

[grid]
max_particles_per_box = {ppb}

[bh]
grav_constant = {gconst!r}
tick_seconds = {dt!r}

[cuda]
threads_per_block = 128

[sequential]
evaluation = com_concat_dedup
force_calculation = numba
"""


def uniform_case(n, seed):
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 2))
    m = 1.0 + rng.random(n)
    return pos[:, 0].copy(), pos[:, 1].copy(), m, np.zeros(n), np.zeros(n)


def two_cluster_case(n, seed):
    """Two tight clusters in opposite corners: most boxes stay empty."""
    rng = np.random.default_rng(seed)
    half = n // 2
    a = 0.02 * rng.random((half, 2))
    b = 1.0 - 0.02 * rng.random((n - half, 2))
    pos = np.concatenate([a, b])
    m = 1.0 + rng.random(n)
    return pos[:, 0].copy(), pos[:, 1].copy(), m, np.zeros(n), np.zeros(n)


def lattice_case(k):
    """(k+1)^2 lattice points on [0,1]^2: many particles sit exactly on box
    edges and on the maximum edge of the bounding box (clipped to G-1)."""
    t = np.arange(k + 1) / k
    xx, yy = np.meshgrid(t, t, indexing="ij")
    n = xx.size
    m = 1.0 + (np.arange(n) % 7) / 7.0
    return xx.ravel().copy(), yy.ravel().copy(), m, np.zeros(n), np.zeros(n)


def duplicate_case(n, seed):
    """Uniform points where every 5th particle duplicates its predecessor's
    position: r^2 = 0 pairs fall under the r^2 <= 1e-5 cutoff."""
    x, y, m, vx, vy = uniform_case(n, seed)
    x[1::5] = x[0:-1:5][: len(x[1::5])]
    y[1::5] = y[0:-1:5][: len(y[1::5])]
    return x, y, m, vx, vy


def moving_case(n, seed):
    """Uniform positions with nonzero initial velocities (like gen_input.py)."""
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 2))
    m = 1.0 + rng.random(n)
    v = (rng.random((n, 2)) - 0.5) * 2.0
    return pos[:, 0].copy(), pos[:, 1].copy(), m, v[:, 0].copy(), v[:, 1].copy()


CASES = {
    # name: (generator, ppb, G const, dt, steps, record steps)
    "c1_uniform10k": (lambda: uniform_case(10_000, 0), 60, 1.0, 1e-4, 10, (0, 9)),
    "n2": (lambda: uniform_case(2, 5), 60, 1.0, 1e-4, 2, (0, 1)),
    "n33": (lambda: uniform_case(33, 6), 4, 1.0, 1e-4, 3, (0, 2)),
    "n1000_g19": (lambda: uniform_case(1000, 7), 4, 1.0, 1e-4, 3, (0, 2)),
    "two_clusters": (lambda: two_cluster_case(600, 8), 3, 1.0, 1e-4, 2, (0, 1)),
    "lattice_edges": (lambda: lattice_case(8), 2, 1.0, 1e-4, 2, (0, 1)),
    "duplicates": (lambda: duplicate_case(400, 9), 5, 1.0, 1e-4, 2, (0, 1)),
    "moving": (lambda: moving_case(2000, 10), 20, 0.5, 1e-3, 5, (0, 4)),
}


def run_case(name, gen, ppb, gconst, dt, nsteps, record):
    import barneshut.internals.particle as p
    from barneshut.internals.config import Config
    from barneshut.implementations.sequential import SequentialBarnesHut

    x, y, m, vx, vy = gen()
    n = len(x)
    with tempfile.NamedTemporaryFile("w", suffix=".ini", delete=False) as f:
        f.write(INI_TEMPLATE.format(ppb=ppb, gconst=gconst, dt=dt))
        ini = f.name
    Config.read_file(ini)
    os.unlink(ini)
    sink = io.StringIO()
    with contextlib.redirect_stdout(sink):
        bh = SequentialBarnesHut()
    bh.n_particles = n
    P = np.zeros((n, p.nfields), dtype=np.float64)
    P[:, p.px], P[:, p.py], P[:, p.mass] = x, y, m
    P[:, p.vx], P[:, p.vy] = vx, vy
    P[:, p.pid] = np.arange(n, dtype=np.float64)
    bh.particles = P

    out = {
        "x0": x, "y0": y, "m": m, "vx0": vx, "vy0": vy,
        "ppb": np.int64(ppb), "gconst": np.float64(gconst), "dt": np.float64(dt),
        "nsteps": np.int64(nsteps), "record_steps": np.array(record, dtype=np.int64),
    }
    t0 = time.time()
    for step in range(nsteps):
        with contextlib.redirect_stdout(sink):
            bh.create_tree()
            bh.summarize()
            bh.evaluate()
        Q = bh.particles
        order = np.argsort(Q[:, p.pid], kind="stable")
        S = Q[order]
        if step in record:
            G = bh.grid_dim
            coms = np.zeros((G, G, 3))
            for i in range(G):
                for j in range(G):
                    c = bh.grid[i][j].cloud.COM
                    coms[i, j] = c.particles[0, :3]
            out[f"s{step}_grid_dim"] = np.int64(G)
            out[f"s{step}_min_xy"] = np.asarray(bh.min_xy, dtype=np.float64)
            out[f"s{step}_max_xy"] = np.asarray(bh.max_xy, dtype=np.float64)
            out[f"s{step}_step"] = np.float64(bh.step)
            out[f"s{step}_gx"] = S[:, p.gx].astype(np.int32)
            out[f"s{step}_gy"] = S[:, p.gy].astype(np.int32)
            out[f"s{step}_coms"] = coms
            out[f"s{step}_ax"] = S[:, p.ax].copy()
            out[f"s{step}_ay"] = S[:, p.ay].copy()
            out[f"s{step}_x"] = S[:, p.px].copy()
            out[f"s{step}_y"] = S[:, p.py].copy()
        # restated tick of the reference GPU path (gpu/grid.py:159-174)
        Q[:, p.vx] += Q[:, p.ax] * dt
        Q[:, p.vy] += Q[:, p.ay] * dt
        Q[:, p.ax] = 0.0
        Q[:, p.ay] = 0.0
        Q[:, p.px] += Q[:, p.vx] * dt
        Q[:, p.py] += Q[:, p.vy] * dt
    order = np.argsort(bh.particles[:, p.pid], kind="stable")
    F = bh.particles[order]
    out["final_x"], out["final_y"] = F[:, p.px].copy(), F[:, p.py].copy()
    out["final_vx"], out["final_vy"] = F[:, p.vx].copy(), F[:, p.vy].copy()
    out["ref_seconds_per_step"] = np.float64((time.time() - t0) / nsteps)
    return out


def main():
    if len(sys.argv) < 2:
        print(__doc__)
        sys.exit(2)
    ref = os.path.abspath(sys.argv[1])
    only = set(sys.argv[2:])
    sys.path.insert(0, os.path.join(HERE, "numba_stub"))
    sys.path.insert(0, ref)
    for name, (gen, ppb, gconst, dt, nsteps, record) in CASES.items():
        if only and name not in only:
            continue
        t0 = time.time()
        out = run_case(name, gen, ppb, gconst, dt, nsteps, record)
        path = os.path.join(HERE, f"ref_{name}.npz")
        np.savez_compressed(path, **out)
        print(f"{name}: n={len(out['x0'])} G={out['s0_grid_dim']} "
              f"{time.time() - t0:.1f}s -> {os.path.basename(path)}", flush=True)


if __name__ == "__main__":
    main()

"""Seeded synthetic particle sets.

The reference measures on files written by ``python-bh/bin/gen_input.py``
(unseeded uniform positions in [0, 499), masses in [0.5, 5), velocities in
(-1, 1)); no dataset ships with it.  These generators stand in for it with
fixed seeds and the shapes of each benchmark configuration:

* ``uniform``          positions U[0,1)^2, masses U[1,2), v = 0
* ``cluster_mixture``  8 isotropic Gaussians (sigma 0.05, centres U[0.2,0.8)^2)
                       plus a 20 % uniform background, clipped to [0, 1 - 2^-24]
* ``batched_systems``  log-uniform sizes in [1024, 262144], uniform or
                       4-cluster layout (50/50), grid ~64 particles per box
* ``gen_input``        the distributions of ``bin/gen_input.py`` ("normal":
                       uniform in [0, 499); "gauss": normal around the centre),
                       seeded

All return float64 arrays (x, y, m, vx, vy).
"""
import math

import numpy as np


def uniform(n, seed=0):
    rng = np.random.default_rng(seed)
    pos = rng.random((n, 2))
    m = 1.0 + rng.random(n)
    z = np.zeros(n)
    return pos[:, 0].copy(), pos[:, 1].copy(), m, z, z.copy()


def cluster_mixture(n, seed=1, nclusters=8, sigma=0.05, background=0.2):
    rng = np.random.default_rng(seed)
    centres = rng.uniform(0.2, 0.8, size=(nclusters, 2))
    is_bg = rng.random(n) < background
    pos = np.empty((n, 2))
    nbg = int(is_bg.sum())
    pos[is_bg] = rng.random((nbg, 2))
    which = rng.integers(0, nclusters, size=n - nbg)
    pos[~is_bg] = centres[which] + rng.normal(0.0, sigma, size=(n - nbg, 2))
    np.clip(pos, 0.0, 1.0 - 2.0 ** -24, out=pos)
    m = rng.uniform(1.0, 2.0, size=n)
    z = np.zeros(n)
    return pos[:, 0].copy(), pos[:, 1].copy(), m, z, z.copy()


def batched_systems(nsys=512, seed=4, nmin=1024, nmax=262144, per_box=64):
    """Returns (list of (x, y, m, vx, vy), list of grid dims)."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(math.log(nmin), math.log(nmax), size=nsys))).astype(np.int64)
    layouts = rng.random(nsys) < 0.5
    systems, grids = [], []
    for s in range(nsys):
        n = int(sizes[s])
        sub = int(rng.integers(0, 2 ** 31))
        if layouts[s]:
            sysd = cluster_mixture(n, seed=sub, nclusters=4, background=0.0)
        else:
            sysd = uniform(n, seed=sub)
        systems.append(sysd)
        grids.append(max(1, int(round(math.sqrt(n / per_box)))))
    return systems, grids


def gen_input(n, distribution="normal", seed=None, domain=500.0):
    """Distributions of python-bh/bin/gen_input.py:35-54, with a seed."""
    rng = np.random.default_rng(seed)
    maxc = domain - 1.0
    if distribution == "normal":
        x = rng.random(n) * maxc
        y = rng.random(n) * maxc
    elif distribution == "gauss":
        x = rng.normal(maxc / 2, maxc / 12, size=n)
        y = rng.normal(maxc / 2, maxc / 12, size=n)
    else:
        raise ValueError(f"unknown distribution {distribution!r}")
    vx = (rng.random(n) - 0.5) * 2.0
    vy = (rng.random(n) - 0.5) * 2.0
    m = 0.5 + rng.random(n) * (5.0 - 0.5)
    return x, y, m, vx, vy


def box_order(x, y, G):
    """Permutation into the order of the state between steps of a running simulation: by box
    key (gx * G + gy) of the square bounding-box grid, within a box quadrant by quadrant (x
    half * 2 + y half, from the key at twice the box resolution), stable within a quadrant."""
    mnx, mny, mxx, mxy = float(x.min()), float(y.min()), float(x.max()), float(y.max())
    xe, ye = mxx - mnx, mxy - mny
    if xe > ye:
        mxy += xe - ye
    elif ye > xe:
        mxx += ye - xe
    step = (mxx - mnx) / G
    if not step > 0:
        return np.arange(len(x))
    kx = np.clip(np.floor((x - mnx) / step), 0, G - 1).astype(np.int64)
    ky = np.clip(np.floor((y - mny) / step), 0, G - 1).astype(np.int64)
    hx = np.clip(np.floor(((x - mnx) / step) * 2.0), 0, 2 * G - 1).astype(np.int64) & 1
    hy = np.clip(np.floor(((y - mny) / step) * 2.0), 0, 2 * G - 1).astype(np.int64) & 1
    return np.argsort(4 * (kx * G + ky) + 2 * hx + hy, kind="stable")


def precision_subsample(n, k=16384, seed=2):
    """Seeded target subsample for force-error measurements."""
    rng = np.random.default_rng(seed + 1000)
    return np.sort(rng.choice(n, size=min(k, n), replace=False))

"""CPU oracle for the 2D grid-decomposition Barnes-Hut step (ctypes wrapper).

TEST INFRASTRUCTURE ONLY.  Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline / reference legs of ``bench.py`` import this module, and only as
the checker or the timed CPU baseline; the product path never calls it.

The C source (``bh_oracle.c``) restates, function by function, the reference's
CPU path (python-bh ``implementations/sequential.py``, ``kernels/grid_decomposition/
sequential/evaluation.py:73-109``, ``kernels/gravity/cpu_numba.py:30-92``,
``kernels/helpers/grid.py``), the tick of its GPU path
(``kernels/grid_decomposition/gpu/grid.py:159-174``), an FP64 direct sum
(``implementations/base.py:16-32``) and an FP64 version of this project's
opening-angle far field.  Parity of the restatement is pinned against golden
vectors produced by the reference itself (``tests/golden/ref_*.npz``).
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "bh_oracle.c")
BUILD_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD_DIR, "liboracle.so")

_lib = None


def build(force=False):
    """Compile bh_oracle.c (no FMA contraction, OpenMP) into _build/liboracle.so."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) >= os.path.getmtime(SRC)):
        return LIB
    tmp = f"{LIB}.{os.getpid()}.tmp"  # concurrent builders never share a temporary
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC",
           "-shared", "-o", tmp, SRC, "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        P = ctypes.POINTER
        d, i, ll, f = ctypes.c_double, ctypes.c_int, ctypes.c_longlong, ctypes.c_float
        pd, pi, pll, pf = P(d), P(i), P(ll), P(f)
        L.oref_grid_dim.argtypes = [ll, i]
        L.oref_grid_dim.restype = i
        L.oref_bbox.argtypes = [ll, pd, pd, i, pd]
        L.oref_keys.argtypes = [ll, pd, pd, i, pd, pi, pi]
        L.oref_reference_evaluate.argtypes = [ll, pd, pd, pd, pd, pd, i, i, d, pd, pd, pi, pi,
                                              pd, pd]
        L.oref_reference_evaluate.restype = i
        L.oref_reference_run.argtypes = [ll, pd, pd, pd, pd, pd, i, i, d, d, i, pd, pd]
        L.oref_reference_run.restype = i
        L.oref_tick.argtypes = [ll, pd, pd, pd, pd, pd, pd, d]
        L.oref_direct.argtypes = [ll, pd, pd, pd, d, d, d, ll, pll, pd, pd, i]
        L.oref_potential.argtypes = [ll, pd, pd, pd, d, d, i]
        L.oref_potential.restype = d
        L.oref_num_levels.argtypes = [i]
        L.oref_num_levels.restype = i
        L.oref_pyramid_cells.argtypes = [i]
        L.oref_pyramid_cells.restype = ll
        L.oref_moments.argtypes = [ll, pd, pd, pd, i, pd, pi, pi, pd, pf]
        L.oref_theta_evaluate.argtypes = [ll, pd, pd, pd, i, i, d, d, d, d, pd, pd, pll, i, i, i,
                                          ctypes.c_void_p]
        L.oref_theta_evaluate.restype = i
        L.oref_theta_evaluate_part.argtypes = [ll, pd, pd, pd, i, i, d, d, d, d, pd, pd, pll, i,
                                               i, i, ctypes.c_void_p, pd, pd]
        L.oref_theta_evaluate_part.restype = i
        L.oref_leaf_moments.argtypes = [ll, pd, pd, pd, i, pd, pd]
        L.oref_gpu_evaluate.argtypes = [ll, pd, pd, pd, i, d, d, i, ctypes.c_void_p, pd, pd, i]
        L.oref_reference_sample_time.argtypes = [ll, pd, pd, pd, i, ll, ll, i, pd]
        _lib = L
    return _lib


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def grid_dim(n, ppb):
    return lib().oref_grid_dim(int(n), int(ppb))


def bbox(x, y, G):
    x, y = _d(x), _d(y)
    out = np.zeros(5)
    lib().oref_bbox(len(x), _p(x), _p(y), int(G), _p(out))
    return out


def keys(x, y, G, bb=None):
    x, y = _d(x), _d(y)
    if bb is None:
        bb = bbox(x, y, G)
    bb = _d(bb)
    kx = np.zeros(len(x), np.int32)
    ky = np.zeros(len(x), np.int32)
    lib().oref_keys(len(x), _p(x), _p(y), int(G), _p(bb), _p(kx, ctypes.c_int),
                    _p(ky, ctypes.c_int))
    return kx, ky


def reference_evaluate(x, y, m, vx=None, vy=None, G=0, ppb=60, gconst=1.0):
    """The reference CPU evaluation (flat far field, r^2 <= 1e-5 cutoff).
    Returns dict(ax, ay, kx, ky, coms[G,G,3], bbox[5], G)."""
    n = len(x)
    x, y, m = _d(x), _d(y), _d(m)
    vx = np.zeros(n) if vx is None else _d(vx)
    vy = np.zeros(n) if vy is None else _d(vy)
    Gd = int(G) if G and G > 0 else grid_dim(n, ppb)
    ax, ay = np.zeros(n), np.zeros(n)
    kx, ky = np.zeros(n, np.int32), np.zeros(n, np.int32)
    coms = np.zeros((Gd, Gd, 3))
    bb = np.zeros(5)
    lib().oref_reference_evaluate(n, _p(x), _p(y), _p(m), _p(vx), _p(vy), Gd, int(ppb),
                                  float(gconst), _p(ax), _p(ay), _p(kx, ctypes.c_int),
                                  _p(ky, ctypes.c_int), _p(coms), _p(bb))
    return dict(ax=ax, ay=ay, kx=kx, ky=ky, coms=coms, bbox=bb, G=Gd)


def reference_run(x, y, m, vx, vy, nsteps, G=0, ppb=60, gconst=1.0, dt=1e-4):
    """nsteps of (reference evaluate, restated tick).  Returns new arrays."""
    x, y, m, vx, vy = (_d(a).copy() for a in (x, y, m, vx, vy))
    n = len(x)
    ax, ay = np.zeros(n), np.zeros(n)
    Gd = lib().oref_reference_run(n, _p(x), _p(y), _p(m), _p(vx), _p(vy), int(G), int(ppb),
                                  float(gconst), float(dt), int(nsteps), _p(ax), _p(ay))
    return dict(x=x, y=y, vx=vx, vy=vy, ax=ax, ay=ay, G=Gd)


def direct(x, y, m, gconst=1.0, eps2=0.0, cutoff=-1.0, targets=None, nthreads=0):
    """FP64 direct sum on the given targets (all particles by default)."""
    x, y, m = _d(x), _d(y), _d(m)
    n = len(x)
    if targets is None:
        t = None
        nt = n
    else:
        t = np.ascontiguousarray(targets, dtype=np.int64)
        nt = len(t)
    ax, ay = np.zeros(nt), np.zeros(nt)
    lib().oref_direct(n, _p(x), _p(y), _p(m), float(gconst), float(eps2), float(cutoff), nt,
                      None if t is None else _p(t, ctypes.c_longlong), _p(ax), _p(ay),
                      int(nthreads))
    return ax, ay


def potential(x, y, m, gconst=1.0, eps2=0.0, nthreads=0):
    x, y, m = _d(x), _d(y), _d(m)
    return lib().oref_potential(len(x), _p(x), _p(y), _p(m), float(gconst), float(eps2),
                                int(nthreads))


def num_levels(G):
    return lib().oref_num_levels(int(G))


def pyramid_cells(G):
    return lib().oref_pyramid_cells(int(G))


def moments(x, y, m, G):
    """Leaf moments + pyramid (FP64) and the float cell records."""
    x, y, m = _d(x), _d(y), _d(m)
    bb = bbox(x, y, G)
    kx, ky = keys(x, y, G, bb)
    nc = pyramid_cells(G)
    mom = np.zeros((nc, 6))
    rec = np.zeros((nc, 4), np.float32)
    lib().oref_moments(len(x), _p(x), _p(y), _p(m), int(G), _p(bb), _p(kx, ctypes.c_int),
                       _p(ky, ctypes.c_int), _p(mom), _p(rec, ctypes.c_float))
    return dict(mom=mom, rec=rec, bbox=bb, kx=kx, ky=ky)


def _mask(n, targets):
    if targets is None:
        return None
    mk = np.zeros(n, np.uint8)
    mk[np.asarray(targets, dtype=np.int64)] = 1
    return mk


def theta_evaluate(x, y, m, G, TG=1, theta=0.5, eps2=0.0, cutoff=0.0, gconst=1.0, nthreads=0,
                   dense_min=0, quad_min=0, targets=None):
    """FP64 opening-angle evaluation (theta <= 0: the reference's flat mode).  dense_min > 0:
    boxes with at least dense_min particles use per-box refined lists; quad_min > 0: boxes with
    at least quad_min particles use per-quadrant refined lists (see bh_oracle.c).  targets (pid
    indices): compute forces only for these (the others stay 0); pair counts cover all targets.
    Returns (ax, ay, n_near_pairs, n_far_pairs) with ax/ay over all n particles."""
    x, y, m = _d(x), _d(y), _d(m)
    n = len(x)
    ax, ay = np.zeros(n), np.zeros(n)
    cnt = np.zeros(2, np.int64)
    mk = _mask(n, targets)
    lib().oref_theta_evaluate(n, _p(x), _p(y), _p(m), int(G), int(TG), float(theta),
                              float(eps2), float(cutoff), float(gconst), _p(ax), _p(ay),
                              _p(cnt, ctypes.c_longlong), int(nthreads), int(dense_min), int(quad_min),
                              None if mk is None else mk.ctypes.data)
    return ax, ay, int(cnt[0]), int(cnt[1])


def theta_evaluate_part(x, y, m, G, bb, leaf, targets, TG=1, theta=0.5, eps2=0.0, cutoff=0.0,
                        gconst=1.0, nthreads=0, dense_min=0, quad_min=0):
    """theta_evaluate on a part of a system (a slab of boxes and the halo boxes its near field
    reaches) with the whole system's square box bb[5] and leaf moments leaf[G, G, 6] given.
    targets: the local indices to evaluate.  Returns (ax, ay, n_near_pairs, n_far_pairs) over the
    local particles (non-targets stay 0) and the targets' pair counts."""
    x, y, m = _d(x), _d(y), _d(m)
    n = len(x)
    ax, ay = np.zeros(n), np.zeros(n)
    cnt = np.zeros(2, np.int64)
    mk = _mask(n, targets)
    bb = _d(bb)
    leaf = _d(leaf).reshape(-1)
    lib().oref_theta_evaluate_part(n, _p(x), _p(y), _p(m), int(G), int(TG), float(theta),
                                   float(eps2), float(cutoff), float(gconst), _p(ax), _p(ay),
                                   _p(cnt, ctypes.c_longlong), int(nthreads), int(dense_min),
                                   int(quad_min), mk.ctypes.data, _p(bb), _p(leaf))
    return ax, ay, int(cnt[0]), int(cnt[1])


def leaf_moments(x, y, m, G, bb):
    """Leaf moments (M, Sx, Sy, Sxx, Sxy, Syy about each box origin), shape (G, G, 6)."""
    x, y, m = _d(x), _d(y), _d(m)
    out = np.zeros((G, G, 6))
    lib().oref_leaf_moments(len(x), _p(x), _p(y), _p(m), int(G), _p(_d(bb)), _p(out))
    return out


def gpu_evaluate(x, y, m, G, gconst=1.0, cutoff=-1.0, skip_zero=False, targets=None, nthreads=0):
    """The reference GPU path's evaluation (gpu/grid.py: flat far field over every box, j != i,
    no cutoff).  skip_zero: drop pairs at distance 0 (which give NaN in the reference GPU path)
    as this project's CUDA path does; cutoff >= 0: also drop pairs with r^2 <= cutoff (1e-5: the
    CPU path's physics).  targets: compute only these (the others stay 0).  Returns (ax, ay)."""
    x, y, m = _d(x), _d(y), _d(m)
    n = len(x)
    ax, ay = np.zeros(n), np.zeros(n)
    mk = _mask(n, targets)
    lib().oref_gpu_evaluate(n, _p(x), _p(y), _p(m), int(G), float(gconst), float(cutoff),
                            int(bool(skip_zero)), None if mk is None else mk.ctypes.data,
                            _p(ax), _p(ay), int(nthreads))
    return ax, ay


def reference_sample_time(x, y, m, G, nsample, nthreads=0, offset=0):
    """Time a bounded sample of one reference CPU step (see bh_oracle.c); nsample >= the
    non-empty boxes times the whole step.  Returns dict(setup_s, sample_s, nonempty, sampled,
    step_s), step_s = setup_s + sample_s * nonempty / sampled."""
    x, y, m = _d(x), _d(y), _d(m)
    out = np.zeros(6)
    lib().oref_reference_sample_time(len(x), _p(x), _p(y), _p(m), int(G), int(nsample),
                                     int(offset), int(nthreads), _p(out))
    return dict(setup_s=out[0], sample_s=out[1], nonempty=int(out[2]), sampled=int(out[3]),
                step_s=out[4])


def tick(x, y, vx, vy, ax, ay, dt):
    x, y, vx, vy = (_d(a).copy() for a in (x, y, vx, vy))
    ax, ay = _d(ax), _d(ay)
    lib().oref_tick(len(x), _p(x), _p(y), _p(vx), _p(vy), _p(ax), _p(ay), float(dt))
    return x, y, vx, vy


def rel_rms(a, b, ax_ref, ay_ref):
    """sqrt(sum |a - a_ref|^2 / sum |a_ref|^2) over 2D vectors."""
    num = np.sum((np.asarray(a) - ax_ref) ** 2 + (np.asarray(b) - ay_ref) ** 2)
    den = np.sum(np.asarray(ax_ref) ** 2 + np.asarray(ay_ref) ** 2)
    return float(np.sqrt(num / den)) if den > 0 else float(np.sqrt(num))

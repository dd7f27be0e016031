"""Parity at the benchmark scales, and the reference GPU path's semantics.

Scales (cluster mixture: 8 Gaussians of sigma 0.05 plus 20 % uniform background, masses in
[1, 2)):
  * N = 1,048,576 on 256 x 256 boxes (seed 1);
  * N = 4,194,304 on 512 x 512 boxes (seed 2), the benchmark's workload.
Both run with the benchmark's tile (4 x 4 target groups, own work items for boxes of >= 16
particles, per-quadrant items for boxes of >= 128), theta = 0.5, softening 1e-4.

Tolerances:
  * box keys per particle: bit-exact against the oracle's restatement of
    sequential.py:32-34 (which implies identical per-box particle sets);
  * near and far pair counts: exact (the same interaction lists as the oracle);
  * accelerations on a seeded 16,384-target subsample: relative RMS <= 1e-5 against the
    FP64 oracle applying the same opening rule (FP32 pairs, compensated far field).

The reference GPU path (kernels/grid_decomposition/gpu/grid.py:116-268; `implementation =
singlegpu`) has no cutoff and skips only the index-identical pair, so two particles at the same
position divide by zero there (NaN).  This project's CUDA path skips every pair at distance 0
instead; elsewhere the two agree.  The oracle restates the reference GPU evaluation
(oracle.gpu_evaluate), and is pinned against the reference CPU path's golden vectors by giving
it the CPU path's cutoff (tests/test_oracle_golden.py).  Tolerance against it: relative RMS
<= 1e-5 (FP32 pairs, FP64 reference).
"""
import configparser

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden_cases

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")

TILE = dict(group_dim=4, dense_min=16, quad_min=128)
SCALES = {"n1m_g256": (1 << 20, 256, 1), "n4m_g512": (1 << 22, 512, 2)}
NSAMPLE = 16384


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def native():
    from barneshut.gb300 import native as n

    return n


def make_plan(n, G, **kw):
    N = native()
    return N.Plan([n], [G], N.make_params(**kw))


@pytest.fixture(scope="module", params=sorted(SCALES))
def system(request):
    from barneshut.gb300 import workloads

    n, G, seed = SCALES[request.param]
    x, y, m, vx, vy = workloads.cluster_mixture(n, seed=seed)
    return request.param, n, G, seed, (x, y, m, vx, vy)


def key_fallback_fraction(p, mn, step, G):
    """Fraction of coordinates whose box key the placement kernel takes from the FP64 quotient:
    the float estimate 2 (float(p) - float(mn)) * float(1 / step), whose error bound tol is
    derived from the system's extent, lies within 2 tol of an integer (k_bbox_finalize and
    half_key1_f32 of the CUDA path, restated here in numpy float32 arithmetic)."""
    am = max(abs(mn[0]), abs(mn[1]))
    tol = 4.0 * ((2.0 * am + G * step) / step + 2.0 * G) * 5.9604644775390625e-8
    tol2 = np.float32(2.0) * np.float32(tol)
    inv_f = np.float32(1.0 / step)
    hits = 0
    for c in range(2):
        q = np.float32(2.0) * ((p[c].astype(np.float32) - np.float32(mn[c])) * inv_f)
        fr = q - np.floor(q)
        hits += int(np.count_nonzero((fr < tol2) | (fr > np.float32(1.0) - tol2)))
    return hits / (2.0 * len(p[0]))


def test_keys_bit_exact_at_scale(system):
    from oracle import oracle

    name, n, G, seed, (x, y, m, vx, vy) = system
    plan = make_plan(n, G, grav_constant=1.0, tick_seconds=1e-5, softening=1e-4, cutoff_r2=0.0,
                     theta=0.5, **TILE)
    plan.load(x, y, m, vx, vy)
    plan.create_tree()
    rec = plan.store_records().cpu().numpy()
    bb = oracle.bbox(x, y, G)
    kx, ky = oracle.keys(x, y, G, bb)
    np.testing.assert_array_equal(rec[:, 9], np.arange(n))
    np.testing.assert_array_equal(rec[:, 7].astype(np.int32), kx)
    np.testing.assert_array_equal(rec[:, 8].astype(np.int32), ky)
    info = plan.grid_info()
    assert info["min_x"] == bb[0] and info["min_y"] == bb[1] and info["step"] == bb[4]
    assert plan.error_flags() == 0
    frac = key_fallback_fraction((x, y), bb[:2], bb[4], G)
    print(f"{name}: FP64 key fallback on {frac:.3%} of coordinates")
    assert frac < 0.01


def test_theta_at_scale(system):
    from oracle import oracle

    name, n, G, seed, (x, y, m, vx, vy) = system
    eps = 1e-4
    plan = make_plan(n, G, grav_constant=1.0, tick_seconds=1e-5, softening=eps, cutoff_r2=0.0,
                     theta=0.5, precision=native().BH_PREC_FP32_KAHAN, **TILE)
    plan.load(x, y, m, vx, vy)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    nn, nf = plan.pair_counts()
    assert plan.error_flags() == 0
    t = np.random.default_rng(seed).choice(n, NSAMPLE, replace=False)
    ax, ay, on, of = oracle.theta_evaluate(x, y, m, G, TG=TILE["group_dim"], theta=0.5,
                                           eps2=eps * eps, cutoff=0.0,
                                           dense_min=TILE["dense_min"],
                                           quad_min=TILE["quad_min"], targets=t)
    assert (nn, nf) == (on, of), "interaction lists differ from the oracle's"
    err = oracle.rel_rms(out["ax"].cpu().numpy()[t], out["ay"].cpu().numpy()[t], ax[t], ay[t])
    print(f"{name}: {nn} near + {nf} far pairs, rel RMS vs FP64 oracle {err:.2e}")
    assert err <= 1e-5, err


# ------------------------------------------------------------ reference GPU semantics
def golden(name):
    return np.load(f"{GOLDEN}/ref_{name}.npz")


SINGLEGPU_KW = dict(tick_seconds=1e-4, softening=0.0, cutoff_r2=0.0, theta=0.0)


@pytest.mark.parametrize("name", golden_cases())
def test_singlegpu_semantics_vs_reference_gpu(name):
    """Flat far field, no cutoff, no softening (the `singlegpu` implementation) against the
    restated reference GPU evaluation on every golden input; where the reference divides by
    zero (particles sharing a position) the CUDA path returns the finite sum without those
    pairs, which the restatement with the distance-0 rule gives."""
    from oracle import oracle

    z = golden(name)
    G = int(z["s0_grid_dim"])
    g = float(z["gconst"])
    plan = make_plan(len(z["x0"]), G, grav_constant=g, **SINGLEGPU_KW)
    plan.load(z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    ax, ay = out["ax"].cpu().numpy(), out["ay"].cpu().numpy()
    assert np.all(np.isfinite(ax)) and np.all(np.isfinite(ay))
    sx, sy = oracle.gpu_evaluate(z["x0"], z["y0"], z["m"], G, gconst=g, skip_zero=True)
    assert oracle.rel_rms(ax, ay, sx, sy) <= 1e-5
    rx, ry = oracle.gpu_evaluate(z["x0"], z["y0"], z["m"], G, gconst=g)
    ok = np.isfinite(rx) & np.isfinite(ry)
    assert oracle.rel_rms(ax[ok], ay[ok], rx[ok], ry[ok]) <= 1e-5
    assert plan.error_flags() == 0


def _singlegpu_run(tmp_path, rounds):
    from barneshut import BarnesHut
    from barneshut.gb300 import particle_io
    import barneshut.internals.particle as p

    z = golden("c1_uniform10k")
    cp = configparser.ConfigParser()
    cp.read(f"{ROOT}/barnes-hut_gb300/configs/parity_c1.ini")
    cp["general"]["implementation"] = "singlegpu"
    cp["general"]["rounds"] = str(rounds)
    cp.remove_option("gb300", "cutoff_r2")  # singlegpu's own default: no cutoff
    ini = tmp_path / f"singlegpu_c1_{rounds}.ini"
    with open(ini, "w") as f:
        cp.write(f)
    inp = tmp_path / "c1.bin"
    particle_io.write_particles(str(inp), z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    bh = BarnesHut(str(ini))
    bh.read_input_file(str(inp))
    bh.run()
    assert bh.bh.grid_dim == int(z["s0_grid_dim"])
    bh.bh.ensure_particles_id_ordered()
    P = bh.bh.get_particles()
    return z, P[:, p.px], P[:, p.py]


def _restated_gpu_rounds(z, rounds):
    from oracle import oracle

    G = int(z["s0_grid_dim"])
    x, y, vx, vy, m = (np.array(z[k], dtype=np.float64) for k in ("x0", "y0", "vx0", "vy0", "m"))
    for _ in range(rounds):
        ax, ay = oracle.gpu_evaluate(x, y, m, G, gconst=float(z["gconst"]), skip_zero=True)
        x, y, vx, vy = oracle.tick(x, y, vx, vy, ax, ay, float(z["dt"]))
    return x, y


def test_singlegpu_dropin_rounds(tmp_path):
    """`implementation = singlegpu` through BarnesHut(ini).run() on the C1 input (N = 10,000,
    16 x 16 boxes, dt = 1e-4) against rounds of the restated reference GPU evaluation with the
    reference GPU tick (gpu/grid.py:159-174).

    With neither cutoff nor softening a pair at distance r feels ~m / r, and the FP32 offsets
    (rounded to 2^-24 of the box edge) give it a relative force error ~2^-24 edge / r (4e-5 at
    r = 1e-4): the few particles with a close partner carry errors far above the typical one,
    and close encounters amplify them over the rounds.  So the rounds are checked in RMS over
    all particles: RMS position error <= 1e-5 of the RMS displacement after one round (the
    accelerations' tolerance: v = 0 initially, so the displacement is a dt^2), and <= 1e-3 after
    ten."""
    def rms_err(z, x, y, rx, ry):
        err = np.sqrt(np.mean((x - rx) ** 2 + (y - ry) ** 2))
        drms = np.sqrt(np.mean((rx - z["x0"]) ** 2 + (ry - z["y0"]) ** 2))
        return err, drms

    z, x1, y1 = _singlegpu_run(tmp_path, 1)
    err, drms = rms_err(z, x1, y1, *_restated_gpu_rounds(z, 1))
    print(f"singlegpu 1 round: RMS error {err:.3e}, RMS displacement {drms:.3e}")
    assert err <= 1e-5 * drms, (err, drms)

    z, x10, y10 = _singlegpu_run(tmp_path, 10)
    rx, ry = _restated_gpu_rounds(z, 10)
    err, drms = rms_err(z, x10, y10, rx, ry)
    print(f"singlegpu 10 rounds: RMS error {err:.3e}, RMS displacement {drms:.3e}, "
          f"max error {max(np.max(np.abs(x10 - rx)), np.max(np.abs(y10 - ry))):.3e}")
    assert err <= 1e-3 * drms, (err, drms)

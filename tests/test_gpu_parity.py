"""Parity of the CUDA path (through the C ABI) with the oracle and with the
reference's own outputs (golden vectors).

Tolerances:
  * box keys, per-box particle sets: bit-exact;
  * flat-mode accelerations vs the reference CPU path: relative RMS <= 1e-5
    (FP32 pair arithmetic, Kahan far field);
  * positions after the stated steps vs the reference: max |dx| <= 2e-7 x the
    largest displacement (unit box; dt = 1e-4, 10 steps; ~1e-9 absolute);
  * theta-mode accelerations vs the FP64 oracle with identical interaction
    lists: relative RMS <= 1e-5 (FP32), 1e-8 (FP64 pairs: the cell centres of
    mass come from FP32 per-warp partial sums accumulated in FP64); pair
    counts exact;
  * two runs of the same step (eager vs graph, fused vs unfused, a second plan on
    the same input): bit-identical -- particles are ordered within a quadrant by
    input order, not by atomic arrival, and every reduction runs in a fixed order;
  * batched vs separate systems: the leaf sums start their 32-particle chunks at
    other offsets, so FP32 sums may differ in the last bits: accelerations and
    velocities within relative RMS 1e-6, positions within 1e-9 absolute.
"""
import numpy as np
import pytest

from conftest import GOLDEN, golden_cases

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def native():
    from barneshut.gb300 import native as n

    return n


def make_plan(n, G, **kw):
    N = native()
    prm = N.make_params(**kw)
    return N.Plan([n] if np.isscalar(n) else n, [G] if np.isscalar(G) else G, prm)


def assert_same_run(oa, ob, sl=slice(None), exact=False):
    from oracle import oracle

    if exact:
        for k in ("x", "y", "vx", "vy", "ax", "ay"):
            np.testing.assert_array_equal(oa[k][sl].cpu().numpy(), ob[k].cpu().numpy(), err_msg=k)
        return
    for k in ("x", "y"):
        d = np.max(np.abs(oa[k][sl].cpu().numpy() - ob[k].cpu().numpy()))
        assert d <= 1e-9, (k, d)
    for a, b in (("vx", "vy"), ("ax", "ay")):
        e = oracle.rel_rms(oa[a][sl].cpu().numpy(), oa[b][sl].cpu().numpy(),
                           ob[a].cpu().numpy(), ob[b].cpu().numpy())
        assert e <= 1e-6, (a, e)


def golden(name):
    return np.load(f"{GOLDEN}/ref_{name}.npz")


REF_KW = dict(grav_constant=1.0, tick_seconds=1e-4, softening=0.0, cutoff_r2=1e-5, theta=0.0)


# ------------------------------------------------------------------ placement
@pytest.mark.parametrize("name", golden_cases())
def test_create_tree_keys_bit_exact(name):
    z = golden(name)
    G = int(z["s0_grid_dim"])
    n = len(z["x0"])
    plan = make_plan(n, G, **REF_KW)
    plan.load(z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    plan.create_tree()
    rec = plan.store_records().cpu().numpy()
    np.testing.assert_array_equal(rec[:, 7].astype(np.int32), z["s0_gx"])
    np.testing.assert_array_equal(rec[:, 8].astype(np.int32), z["s0_gy"])
    np.testing.assert_array_equal(rec[:, 9], np.arange(n))
    info = plan.grid_info()
    assert info["min_x"] == z["s0_min_xy"][0] and info["min_y"] == z["s0_min_xy"][1]
    assert info["step"] == z["s0_step"]
    assert plan.error_flags() == 0


@pytest.mark.parametrize("name", golden_cases())
def test_summarize_coms(name):
    z = golden(name)
    G = int(z["s0_grid_dim"])
    plan = make_plan(len(z["x0"]), G, **REF_KW)
    plan.load(z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    plan.create_tree()
    plan.summarize()
    c = plan.box_moments().cpu().numpy()
    ref = z["s0_coms"]
    np.testing.assert_array_equal(c[..., 2] > 0, ref[..., 2] > 0)
    np.testing.assert_allclose(c[..., 2], ref[..., 2], rtol=1e-6)
    # centres of mass: FP32 per-particle products, FP64 accumulation
    step = float(z["s0_step"])
    assert np.max(np.abs(c[..., :2] - ref[..., :2])) <= 1e-6 * step


# ---------------------------------------------------------------- evaluation
@pytest.mark.parametrize("name", golden_cases())
def test_flat_forces_vs_reference(name):
    z = golden(name)
    G = int(z["s0_grid_dim"])
    plan = make_plan(len(z["x0"]), G, **dict(REF_KW, grav_constant=float(z["gconst"])))
    plan.load(z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    ax, ay = out["ax"].cpu().numpy(), out["ay"].cpu().numpy()
    from oracle import oracle

    err = oracle.rel_rms(ax, ay, z["s0_ax"], z["s0_ay"])
    assert err <= 1e-5, err


def test_c1_ten_steps_positions():
    """C1: 10 fused steps (create_tree, summarize, evaluate + tick) vs the
    reference driven with the restated tick."""
    z = golden("c1_uniform10k")
    G = int(z["s0_grid_dim"])
    plan = make_plan(len(z["x0"]), G, **REF_KW)
    plan.load(z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"])
    plan.step(int(z["nsteps"]))
    out = plan.store()
    from oracle import oracle

    dx = np.max(np.abs(out["x"].cpu().numpy() - z["final_x"]))
    dy = np.max(np.abs(out["y"].cpu().numpy() - z["final_y"]))
    # FP32 forces (~1e-7 relative) move positions by ~1e-7 of the displacement
    disp = max(np.max(np.abs(z["final_x"] - z["x0"])), np.max(np.abs(z["final_y"] - z["y0"])))
    assert max(dx, dy) <= 2e-7 * disp, (dx, dy, disp)
    err = oracle.rel_rms(out["ax"].cpu().numpy(), out["ay"].cpu().numpy(), z["s9_ax"], z["s9_ay"])
    assert err <= 1e-5, err


def test_unfused_phases_equal_fused():
    from barneshut.gb300 import workloads

    x, y, m, vx, vy = workloads.uniform(3000, seed=21)
    a = make_plan(3000, 8, **REF_KW)
    b = make_plan(3000, 8, **REF_KW)
    a.load(x, y, m, vx, vy)
    b.load(x, y, m, vx, vy)
    for _ in range(3):
        a.create_tree()
        a.summarize()
        a.evaluate()
        a.timestep()
    b.step(3)
    a.create_tree()
    a.summarize()
    a.evaluate()
    b.create_tree()
    b.summarize()
    b.evaluate()
    assert_same_run(a.store(), b.store(), exact=True)


# ---------------------------------------------------------------- theta mode
@pytest.mark.parametrize("theta,TG,G", [(0.3, 1, 16), (0.5, 2, 16), (0.5, 4, 19), (0.8, 2, 32)])
@pytest.mark.parametrize("prec", [0, 1, 2])
@pytest.mark.parametrize("walk", [False, True], ids=["lists", "walk"])
def test_theta_vs_fp64_oracle(theta, TG, G, prec, walk):
    """Both theta-mode force paths -- interaction lists built once per group and streamed (the
    default for FP32 pairs), and the pyramid walk inside the force kernel (BH_FLAG_WALK; always
    used for FP64 pairs) -- against the FP64 oracle with the same opening rule."""
    from barneshut.gb300 import workloads
    from oracle import oracle

    if walk and prec == 2:
        pytest.skip("FP64 pairs always walk")
    x, y, m, vx, vy = workloads.cluster_mixture(20000, seed=31)
    eps = 1e-3
    plan = make_plan(20000, G, grav_constant=1.0, tick_seconds=1e-5, softening=eps, cutoff_r2=0.0,
                     theta=theta, group_dim=TG, precision=prec,
                     flags=native().BH_FLAG_WALK if walk else 0)
    plan.load(x, y, m, vx, vy)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    nn, nf = plan.pair_counts()
    # list streaming refines the near lists of dense boxes; the walk keeps the group lists
    walking = walk or prec == 2
    dense = 0 if walking else native().BH_STREAM_DENSE_MIN
    quad = 0 if walking else native().BH_STREAM_QUAD_MIN
    ax, ay, on, of = oracle.theta_evaluate(x, y, m, G, TG=TG, theta=theta, eps2=eps * eps, cutoff=0.0,
                                           dense_min=dense, quad_min=quad)
    assert (nn, nf) == (on, of), "interaction lists differ from the oracle's"
    err = oracle.rel_rms(out["ax"].cpu().numpy(), out["ay"].cpu().numpy(), ax, ay)
    assert err <= (1e-8 if prec == 2 else 1e-5), err
    assert plan.error_flags() == 0


@pytest.mark.parametrize("prec", [0, 1])
@pytest.mark.parametrize("walk", [False, True], ids=["lists", "walk"])
def test_alternative_builds_vs_fp64_oracle(prec, walk):
    """The force kernels' other builds (tune = 1: list streaming on 8 CTAs per SM with 64
    registers and 88-source passes; the walk on 6 CTAs per SM), which the autotuner times, give
    the oracle's interaction lists and forces like the default builds."""
    from barneshut.gb300 import workloads
    from oracle import oracle

    x, y, m, vx, vy = workloads.cluster_mixture(20000, seed=33)
    eps, theta, TG, G = 1e-3, 0.5, 4, 19
    plan = make_plan(20000, G, grav_constant=1.0, tick_seconds=1e-5, softening=eps, cutoff_r2=0.0,
                     theta=theta, group_dim=TG, precision=prec, tune=1,
                     flags=native().BH_FLAG_WALK if walk else 0)
    plan.load(x, y, m, vx, vy)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    nn, nf = plan.pair_counts()
    dense = 0 if walk else native().BH_STREAM_DENSE_MIN
    quad = 0 if walk else native().BH_STREAM_QUAD_MIN
    ax, ay, on, of = oracle.theta_evaluate(x, y, m, G, TG=TG, theta=theta, eps2=eps * eps, cutoff=0.0,
                                           dense_min=dense, quad_min=quad)
    assert (nn, nf) == (on, of), "interaction lists differ from the oracle's"
    err = oracle.rel_rms(out["ax"].cpu().numpy(), out["ay"].cpu().numpy(), ax, ay)
    assert err <= 1e-5, err
    assert plan.error_flags() == 0


@pytest.mark.parametrize("TG,dense_min,quad_min", [(2, 16, 32), (4, 8, 24), (4, 16, -1)])
def test_refined_lists_vs_fp64_oracle(TG, dense_min, quad_min):
    """List streaming with per-box and per-quadrant refinement thresholds low enough that many
    boxes of a 16 x 16 grid take each path: pair counts exact, forces within 1e-5 of the oracle
    applying the same rule (quad_min < 0: no quadrant refinement)."""
    from barneshut.gb300 import workloads
    from oracle import oracle

    x, y, m, vx, vy = workloads.cluster_mixture(20000, seed=33)
    eps = 1e-3
    plan = make_plan(20000, 16, grav_constant=1.0, tick_seconds=1e-5, softening=eps, cutoff_r2=0.0,
                     theta=0.5, group_dim=TG, precision=1, dense_min=dense_min, quad_min=quad_min)
    plan.load(x, y, m, vx, vy)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    nn, nf = plan.pair_counts()
    ax, ay, on, of = oracle.theta_evaluate(x, y, m, 16, TG=TG, theta=0.5, eps2=eps * eps, cutoff=0.0,
                                           dense_min=dense_min, quad_min=max(quad_min, 0))
    assert (nn, nf) == (on, of)
    assert oracle.rel_rms(out["ax"].cpu().numpy(), out["ay"].cpu().numpy(), ax, ay) <= 1e-5
    assert plan.error_flags() == 0


@pytest.mark.parametrize("TG,G,dense_min", [(4, 128, 8), (8, 96, 4)])
def test_sparse_boxes_many_descriptors_per_pass(TG, G, dense_min):
    """One or two particles per box: a staging pass of the list-streaming kernel spans more than
    a warp's worth (32) of near-box descriptors, on group lists and on refined lists alike.  Pair
    counts exact, forces within 1e-5 of the oracle, and every bounded copy wait completes."""
    from barneshut.gb300 import workloads
    from oracle import oracle

    x, y, m, vx, vy = workloads.cluster_mixture(20000, seed=35)
    eps = 1e-3
    plan = make_plan(20000, G, grav_constant=1.0, tick_seconds=1e-5, softening=eps, cutoff_r2=0.0,
                     theta=0.5, group_dim=TG, precision=1, dense_min=dense_min, quad_min=-1)
    plan.load(x, y, m, vx, vy)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    assert plan.error_flags() == 0
    nn, nf = plan.pair_counts()
    ax, ay, on, of = oracle.theta_evaluate(x, y, m, G, TG=TG, theta=0.5, eps2=eps * eps, cutoff=0.0,
                                           dense_min=dense_min, quad_min=0)
    assert (nn, nf) == (on, of)
    assert oracle.rel_rms(out["ax"].cpu().numpy(), out["ay"].cpu().numpy(), ax, ay) <= 1e-5


def test_theta_error_vs_direct_sum():
    from barneshut.gb300 import workloads
    from oracle import oracle

    x, y, m, vx, vy = workloads.cluster_mixture(30000, seed=32)
    plan = make_plan(30000, 32, grav_constant=1.0, softening=1e-3, cutoff_r2=0.0, theta=0.5)
    plan.load(x, y, m, vx, vy)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    t = np.arange(0, 30000, 7)
    dax, day = oracle.direct(x, y, m, eps2=1e-6, cutoff=0.0, targets=t)
    err = oracle.rel_rms(out["ax"].cpu().numpy()[t], out["ay"].cpu().numpy()[t], dax, day)
    assert err < 5e-3, err


# ---------------------------------------------------------------- edge cases
@pytest.mark.parametrize("n", [1, 2, 33])
def test_tiny_systems(n):
    from barneshut.gb300 import workloads
    from oracle import oracle

    x, y, m, vx, vy = workloads.uniform(n, seed=40 + n)
    plan = make_plan(n, 4 if n > 2 else 1, **REF_KW)
    plan.load(x, y, m, vx, vy)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    if n == 1:
        assert out["ax"].item() == 0.0 and out["ay"].item() == 0.0
    else:
        r = oracle.reference_evaluate(x, y, m, G=4 if n > 2 else 1, gconst=1.0)
        assert oracle.rel_rms(out["ax"].cpu().numpy(), out["ay"].cpu().numpy(), r["ax"], r["ay"]) < 1e-5
    assert plan.error_flags() == 0


def test_all_coincident_points():
    n = 64
    x = np.full(n, 0.25)
    y = np.full(n, 0.75)
    m = np.ones(n)
    z = np.zeros(n)
    plan = make_plan(n, 4, **REF_KW)
    plan.load(x, y, m, z, z)
    plan.step(2)
    out = plan.store()
    assert np.all(out["ax"].cpu().numpy() == 0.0)
    np.testing.assert_array_equal(out["x"].cpu().numpy(), x)
    assert plan.error_flags() == 0


def test_nan_position_raises_flag():
    from barneshut.gb300 import workloads

    N = native()
    x, y, m, vx, vy = workloads.uniform(1000, seed=50)
    x[17] = np.nan
    plan = make_plan(1000, 4, **REF_KW)
    plan.load(x, y, m, vx, vy)
    plan.create_tree()
    flags = plan.error_flags(raise_on_error=False)
    assert flags & N.BH_DEV_NAN_POSITION
    assert plan.error_flags(raise_on_error=False) == 0  # cleared


# ---------------------------------------------------------------- batching / graphs
@pytest.mark.parametrize("sizes", [(1500, 5000, 700), (1501, 4999, 703)], ids=["aligned", "ragged"])
def test_batched_equals_separate(sizes):
    """Systems stepped together equal each system stepped alone; the ragged sizes put system
    boundaries inside a placement thread's four particles and inside 32-particle leaf chunks."""
    from barneshut.gb300 import workloads

    systems = [workloads.uniform(sizes[0], seed=60), workloads.cluster_mixture(sizes[1], seed=61),
               workloads.uniform(sizes[2], seed=62)]
    grids = [5, 9, 3]
    kw = dict(grav_constant=1.0, tick_seconds=1e-5, softening=1e-3, cutoff_r2=0.0, theta=0.5,
              group_dim=2)
    plan = make_plan([len(s[0]) for s in systems], grids, **kw)
    cat = [np.concatenate([s[k] for s in systems]) for k in range(5)]
    plan.load(*cat)
    plan.step(3)
    allout = plan.store()
    off = 0
    for s, G in zip(systems, grids):
        p1 = make_plan(len(s[0]), G, **kw)
        p1.load(*s)
        p1.step(3)
        o1 = p1.store()
        n = len(s[0])
        assert_same_run(allout, o1, slice(off, off + n))
        off += n


@pytest.mark.parametrize("theta", [0.5, 0.0])
def test_step_bit_reproducible_n1m(theta):
    """Two plans on the same N = 1,048,576 cluster mixture (256 x 256 boxes), from the caller's
    particle order, three steps each (graph replays): positions, velocities and accelerations
    bit-identical.  theta 0.5: list streaming with quadrant items; theta 0: the reference's flat
    far field (the walk).  Quadrants hold up to about seventy particles here, so both the
    in-register and the shared-memory paths of the quadrant sort run."""
    from barneshut.gb300 import workloads

    x, y, m, vx, vy = workloads.cluster_mixture(1 << 20, seed=1)
    if theta > 0:
        kw = dict(grav_constant=1.0, tick_seconds=1e-5, softening=1e-4, cutoff_r2=0.0, theta=0.5,
                  group_dim=4, dense_min=16, quad_min=128)
    else:
        kw = dict(REF_KW, tick_seconds=1e-5)
    outs = []
    for _ in range(2):
        plan = make_plan(1 << 20, 256, **kw)
        plan.load(x, y, m, vx, vy)
        plan.step_graph(3)
        outs.append(plan.store())
        assert plan.error_flags() == 0
        plan.close()
    assert_same_run(outs[0], outs[1], exact=True)


def test_long_quadrants_sorted():
    """Ten thousand particles in one box (a 1 x 1 grid) and a few hundred in others: the quadrant
    sort's CTA paths (bitonic up to 4,096 entries, radix beyond) give the same step as a second
    plan, and the step matches the oracle's flat evaluation."""
    from barneshut.gb300 import workloads
    from oracle import oracle

    rng = np.random.default_rng(77)
    n = 40000
    x = np.concatenate([rng.normal(0.3, 0.01, n // 2), rng.random(n // 2)])
    y = np.concatenate([rng.normal(0.3, 0.01, n // 2), rng.random(n // 2)])
    m = rng.uniform(1, 2, n)
    z = np.zeros(n)
    outs = []
    for _ in range(2):
        plan = make_plan(n, 8, **REF_KW)
        plan.load(x, y, m, z, z)
        plan.create_tree()
        plan.summarize()
        plan.evaluate()
        outs.append(plan.store())
        rec = plan.store_records().cpu().numpy()
        kx, ky = oracle.keys(x, y, 8)
        np.testing.assert_array_equal(rec[:, 7].astype(np.int32), kx)
        np.testing.assert_array_equal(rec[:, 8].astype(np.int32), ky)
        plan.close()
    assert_same_run(outs[0], outs[1], exact=True)
    ref = oracle.reference_evaluate(x, y, m, G=8, gconst=1.0)
    assert oracle.rel_rms(outs[0]["ax"].cpu().numpy(), outs[0]["ay"].cpu().numpy(),
                          ref["ax"], ref["ay"]) <= 1e-5


def test_accelerations_zero_until_evaluated():
    """A load writes no accelerations: until an evaluation they read as zero (store), and a tick
    right after the load moves the particles by their velocities alone (gpu/grid.py:159-174 with
    a = 0), also after an earlier step left accelerations in the plan."""
    from barneshut.gb300 import workloads

    x, y, m, vx, vy = workloads.uniform(2000, seed=72)
    plan = make_plan(2000, 8, **REF_KW)
    plan.load(x, y, m, vx, vy)
    plan.step(1)  # leaves non-zero accelerations behind
    plan.load(x, y, m, vx, vy)
    o = plan.store()
    assert not o["ax"].any() and not o["ay"].any()
    plan.timestep()
    o = plan.store()
    dt = REF_KW["tick_seconds"]
    # (the device may fuse x + v dt into one rounding)
    np.testing.assert_allclose(o["x"].cpu().numpy(), x + vx * dt, rtol=0, atol=1e-15)
    np.testing.assert_allclose(o["y"].cpu().numpy(), y + vy * dt, rtol=0, atol=1e-15)
    assert not o["ax"].any()


def test_summarize_after_set_leaf_moments():
    """The leaf sums come with the scatter (k_gather); after bh_set_leaf_moments overwrote them,
    bh_summarize sums the leaves from the particles again (the stand-alone leaf pass): the leaf
    moments and the step equal those of a plan that never had them replaced, bit for bit.  Boxes
    of 1 to ~600 particles cover single-chunk boxes and boxes over many chunks."""
    from barneshut.gb300 import workloads

    x, y, m, vx, vy = workloads.cluster_mixture(30000, seed=71)
    kw = dict(grav_constant=1.0, tick_seconds=1e-5, softening=1e-3, cutoff_r2=0.0, theta=0.5)
    a = make_plan(30000, 16, **kw)
    b = make_plan(30000, 16, **kw)
    for p in (a, b):
        p.load(x, y, m, vx, vy)
        p.create_tree()
    a.summarize()
    b.set_leaf_moments(torch.full((16, 16, 6), 3.0, dtype=torch.float64, device="cuda"))
    b.summarize()
    la, lb = a.leaf_moments(), b.leaf_moments()
    assert torch.equal(la, lb)
    assert la[..., 0].sum().item() == pytest.approx(float(np.sum(m)), rel=1e-6)
    a.evaluate()
    b.evaluate()
    assert_same_run(a.store(), b.store(), exact=True)


def test_graph_replay_equals_eager():
    from barneshut.gb300 import workloads

    x, y, m, vx, vy = workloads.cluster_mixture(8000, seed=70)
    kw = dict(grav_constant=1.0, tick_seconds=1e-5, softening=1e-3, cutoff_r2=0.0, theta=0.5)
    a = make_plan(8000, 16, **kw)
    b = make_plan(8000, 16, **kw)
    a.load(x, y, m, vx, vy)
    b.load(x, y, m, vx, vy)
    a.step(4)
    b.step_graph(2)
    b.step_graph(2)
    assert_same_run(a.store(), b.store(), exact=True)


@pytest.mark.parametrize("case", ["stream", "stream_quad", "walk", "flat", "batched"])
def test_kernels_per_step_matches_graph(case):
    """bh_kernels_per_step (the launch count the benchmark reports) equals the kernel nodes of
    the captured step graph, nsteps rounds at a time."""
    from barneshut.gb300 import workloads

    N = native()
    x, y, m, vx, vy = workloads.cluster_mixture(30000, seed=71)
    kw = dict(grav_constant=1.0, tick_seconds=1e-5, softening=1e-3, cutoff_r2=0.0, theta=0.5)
    n, G = [30000], [32]
    if case == "stream_quad":
        kw.update(group_dim=2, dense_min=16, quad_min=32)
    elif case == "walk":
        kw.update(flags=N.BH_FLAG_WALK)
    elif case == "flat":
        kw.update(theta=0.0, softening=0.0, cutoff_r2=1e-5)
    elif case == "batched":
        n, G = [20000, 10000], [24, 4]
    plan = make_plan(n, G, **kw)
    plan.load(x, y, m, vx, vy)
    for nsteps in (1, 3):
        plan.step_graph(nsteps)
        assert plan.graph_kernel_nodes() == nsteps * plan.kernels_per_step()
    assert plan.error_flags() == 0


# ---------------------------------------------------------------- samplers
def test_direct_sample_matches_oracle():
    from barneshut.gb300 import workloads
    from oracle import oracle

    x, y, m, vx, vy = workloads.uniform(4000, seed=80)
    plan = make_plan(4000, 8, grav_constant=2.0, softening=1e-3, cutoff_r2=0.0, theta=0.5)
    plan.load(x, y, m, vx, vy)
    plan.step(1)  # state is box-sorted now; the sampler must map pids
    st = plan.store()
    xs, ys = st["x"].cpu().numpy(), st["y"].cpu().numpy()
    t = np.array([0, 5, 999, 3999])
    ax, ay = plan.direct_sample(t)
    rax, ray = oracle.direct(xs, ys, m, gconst=2.0, eps2=1e-6, cutoff=-1.0, targets=t)
    np.testing.assert_allclose(ax.cpu().numpy(), rax, rtol=1e-10)
    np.testing.assert_allclose(ay.cpu().numpy(), ray, rtol=1e-10)


def test_diagnostics_energy_momentum():
    from barneshut.gb300 import workloads
    from oracle import oracle

    x, y, m, vx, vy = workloads.gen_input(1500, "normal", seed=3)
    plan = make_plan(1500, 8, grav_constant=1.0, softening=1e-2, cutoff_r2=0.0, theta=0.5)
    plan.load(x, y, m, vx, vy)
    ke, px, py, pe = plan.diagnostics(potential=True)
    assert abs(ke - 0.5 * np.sum(m * (vx ** 2 + vy ** 2))) < 1e-10 * ke
    assert abs(px - np.sum(m * vx)) < 1e-9 * np.sum(np.abs(m * vx))
    ref_pe = oracle.potential(x, y, m, 1.0, 1e-4)
    assert abs(pe - ref_pe) < 1e-9 * abs(ref_pe)

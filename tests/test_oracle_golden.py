"""The oracle (oracle/bh_oracle.c) against golden vectors produced by the
reference CPU path itself (tests/golden/make_golden.py)."""
import numpy as np
import pytest

from conftest import GOLDEN, golden_cases

CASES = golden_cases()


def load(name):
    return np.load(f"{GOLDEN}/ref_{name}.npz")


def test_golden_present():
    assert "c1_uniform10k" in CASES, "C1 golden vectors missing"
    assert len(CASES) >= 7


@pytest.mark.parametrize("name", CASES)
def test_grid_bbox_keys_coms_bit_exact(oracle_mod, name):
    z = load(name)
    for s in z["record_steps"]:
        s = int(s)
        G = int(z[f"s{s}_grid_dim"])
        if s == 0:
            x, y, m = z["x0"], z["y0"], z["m"]
        else:
            x, y = z[f"s{s}_x"], z[f"s{s}_y"]
            m = z["m"]
        assert oracle_mod.grid_dim(len(x), int(z["ppb"])) == G
        r = oracle_mod.reference_evaluate(x, y, m, G=G, ppb=int(z["ppb"]), gconst=float(z["gconst"]))
        np.testing.assert_array_equal(r["bbox"][:2], z[f"s{s}_min_xy"])
        assert r["bbox"][4] == z[f"s{s}_step"]
        np.testing.assert_array_equal(r["kx"], z[f"s{s}_gx"])
        np.testing.assert_array_equal(r["ky"], z[f"s{s}_gy"])
        np.testing.assert_array_equal(r["coms"], z[f"s{s}_coms"])


@pytest.mark.parametrize("name", CASES)
def test_accelerations_match_reference(oracle_mod, name):
    z = load(name)
    for s in z["record_steps"]:
        s = int(s)
        G = int(z[f"s{s}_grid_dim"])
        x, y = (z["x0"], z["y0"]) if s == 0 else (z[f"s{s}_x"], z[f"s{s}_y"])
        r = oracle_mod.reference_evaluate(x, y, z["m"], G=G, ppb=int(z["ppb"]),
                                          gconst=float(z["gconst"]))
        err = oracle_mod.rel_rms(r["ax"], r["ay"], z[f"s{s}_ax"], z[f"s{s}_ay"])
        assert err < 1e-13, (name, s, err)


@pytest.mark.parametrize("name", CASES)
def test_multistep_positions_match_reference(oracle_mod, name):
    z = load(name)
    if name == "c1_uniform10k":
        pytest.skip("covered by the CPU-budget-friendly 2-step check below")
    r = oracle_mod.reference_run(z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"], int(z["nsteps"]),
                                 ppb=int(z["ppb"]), gconst=float(z["gconst"]), dt=float(z["dt"]))
    assert np.max(np.abs(r["x"] - z["final_x"])) < 1e-12
    assert np.max(np.abs(r["y"] - z["final_y"])) < 1e-12
    assert np.max(np.abs(r["vx"] - z["final_vx"])) <= 1e-9 * max(1.0, np.max(np.abs(z["final_vx"])))


def test_c1_ten_steps(oracle_mod):
    z = load("c1_uniform10k")
    r = oracle_mod.reference_run(z["x0"], z["y0"], z["m"], z["vx0"], z["vy0"], int(z["nsteps"]),
                                 ppb=int(z["ppb"]), gconst=float(z["gconst"]), dt=float(z["dt"]))
    assert np.max(np.abs(r["x"] - z["final_x"])) < 1e-12
    assert np.max(np.abs(r["y"] - z["final_y"])) < 1e-12
    last = int(z["record_steps"][-1])
    err = oracle_mod.rel_rms(r["ax"], r["ay"], z[f"s{last}_ax"], z[f"s{last}_ay"])
    assert err < 1e-12


@pytest.mark.parametrize("name", CASES)
def test_theta_oracle_flat_mode_is_reference(oracle_mod, name):
    """theta <= 0 in the opening-angle oracle reproduces the reference."""
    z = load(name)
    G = int(z["s0_grid_dim"])
    ax, ay, nn, nf = oracle_mod.theta_evaluate(z["x0"], z["y0"], z["m"], G, TG=1, theta=0.0,
                                               eps2=0.0, cutoff=1e-5, gconst=float(z["gconst"]))
    assert oracle_mod.rel_rms(ax, ay, z["s0_ax"], z["s0_ay"]) < 1e-13


# ------------------------------------------------ the reference GPU path's semantics
@pytest.mark.parametrize("name", CASES)
def test_gpu_restatement_pinned_to_reference_cpu(oracle_mod, name):
    """The restatement of the reference GPU evaluation (gpu/grid.py: every box in (gx, gy) order,
    j != i, COMs of all other boxes) reproduces the reference CPU path's golden accelerations
    when given the CPU path's r^2 <= 1e-5 cutoff: the two paths differ only in that cutoff."""
    z = load(name)
    G = int(z["s0_grid_dim"])
    ax, ay = oracle_mod.gpu_evaluate(z["x0"], z["y0"], z["m"], G, gconst=float(z["gconst"]),
                                     cutoff=1e-5)
    assert oracle_mod.rel_rms(ax, ay, z["s0_ax"], z["s0_ay"]) < 1e-13


@pytest.mark.parametrize("name", CASES)
def test_gpu_restatement_coincident_rule(oracle_mod, name):
    """Without a cutoff the reference GPU path gives NaN exactly for particles that share their
    position with another particle (dist = 0 between different pids); everywhere else its result
    equals the rule of this project's CUDA path (pairs at distance 0 skipped), which in turn is
    the opening-angle oracle's flat mode with cutoff 0."""
    z = load(name)
    G = int(z["s0_grid_dim"])
    x, y, m, g = z["x0"], z["y0"], z["m"], float(z["gconst"])
    rx, ry = oracle_mod.gpu_evaluate(x, y, m, G, gconst=g)
    sx, sy = oracle_mod.gpu_evaluate(x, y, m, G, gconst=g, skip_zero=True)
    pos = np.stack([x, y], 1)
    _, inv, cnt = np.unique(pos, axis=0, return_inverse=True, return_counts=True)
    shared = cnt[inv.ravel()] > 1
    bad = ~(np.isfinite(rx) & np.isfinite(ry))
    np.testing.assert_array_equal(bad, shared)
    np.testing.assert_array_equal(rx[~bad], sx[~bad])
    np.testing.assert_array_equal(ry[~bad], sy[~bad])
    assert np.all(np.isfinite(sx)) and np.all(np.isfinite(sy))
    tx, ty, _, _ = oracle_mod.theta_evaluate(x, y, m, G, TG=1, theta=0.0, eps2=0.0, cutoff=0.0,
                                             gconst=g)
    assert oracle_mod.rel_rms(sx, sy, tx, ty) < 1e-13
    if name == "duplicates":
        assert shared.sum() > 0


def test_theta_oracle_target_mask(oracle_mod):
    """Forces restricted to a target subset equal the full evaluation on that subset; pair counts
    always cover every target."""
    z = load("two_clusters")
    G = int(z["s0_grid_dim"])
    t = np.arange(0, len(z["x0"]), 7)
    full = oracle_mod.theta_evaluate(z["x0"], z["y0"], z["m"], G, TG=2, theta=0.5, eps2=1e-6,
                                     dense_min=8, quad_min=16)
    sub = oracle_mod.theta_evaluate(z["x0"], z["y0"], z["m"], G, TG=2, theta=0.5, eps2=1e-6,
                                    dense_min=8, quad_min=16, targets=t)
    assert full[2:] == sub[2:]
    np.testing.assert_array_equal(full[0][t], sub[0][t])
    np.testing.assert_array_equal(full[1][t], sub[1][t])
    rest = np.setdiff1d(np.arange(len(z["x0"])), t)
    assert np.all(sub[0][rest] == 0.0)

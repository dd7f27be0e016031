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

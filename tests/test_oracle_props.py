"""Properties of the oracle beyond the golden vectors."""
import numpy as np
import pytest

from barneshut.gb300 import workloads


def test_direct_sum_antisymmetry_momentum(oracle_mod):
    x, y, m, _, _ = workloads.uniform(500, seed=3)
    ax, ay = oracle_mod.direct(x, y, m, eps2=1e-6, cutoff=0.0)
    # total force sum_i m_i a_i = 0 (Newton's third law)
    assert abs(np.sum(m * ax)) < 1e-9 * np.sum(np.abs(m * ax))
    assert abs(np.sum(m * ay)) < 1e-9 * np.sum(np.abs(m * ay))


@pytest.mark.parametrize("theta,TG", [(0.3, 1), (0.5, 2), (0.8, 4)])
def test_theta_error_shrinks_with_theta(oracle_mod, theta, TG):
    x, y, m, _, _ = workloads.cluster_mixture(3000, seed=5)
    dax, day = oracle_mod.direct(x, y, m, eps2=1e-6, cutoff=0.0)
    ax, ay, nn, nf = oracle_mod.theta_evaluate(x, y, m, 16, TG=TG, theta=theta, eps2=1e-6)
    err = oracle_mod.rel_rms(ax, ay, dax, day)
    assert err < {0.3: 3e-3, 0.5: 1e-2, 0.8: 3e-2}[theta]
    assert nn > 0 and nf > 0


@pytest.mark.parametrize("TG", [2, 4])
def test_dense_box_refinement(oracle_mod, TG):
    """Per-box (and per-quadrant) refinement of dense boxes' near lists moves near pairs to far
    entries, keeps the error within the opening-angle bound, and is the identity when no box is
    dense."""
    x, y, m, _, _ = workloads.cluster_mixture(20000, seed=7)
    dax, day = oracle_mod.direct(x, y, m, eps2=1e-6, cutoff=0.0)
    a0 = oracle_mod.theta_evaluate(x, y, m, 16, TG=TG, theta=0.5, eps2=1e-6)
    a1 = oracle_mod.theta_evaluate(x, y, m, 16, TG=TG, theta=0.5, eps2=1e-6, dense_min=64)
    a2 = oracle_mod.theta_evaluate(x, y, m, 16, TG=TG, theta=0.5, eps2=1e-6, dense_min=10 ** 9)
    a3 = oracle_mod.theta_evaluate(x, y, m, 16, TG=TG, theta=0.5, eps2=1e-6, dense_min=64, quad_min=64)
    assert a1[2] < a0[2] and a1[3] > a0[3]
    assert a3[2] < a1[2] and a3[3] > a1[3]  # quadrants refine further
    assert a2[2:] == a0[2:] and np.array_equal(a2[0], a0[0])
    assert oracle_mod.rel_rms(a1[0], a1[1], dax, day) < 1e-3
    assert oracle_mod.rel_rms(a3[0], a3[1], dax, day) < 1e-3


def test_theta_tiny_is_direct(oracle_mod):
    x, y, m, _, _ = workloads.uniform(800, seed=4)
    dax, day = oracle_mod.direct(x, y, m, eps2=1e-6, cutoff=0.0)
    ax, ay, nn, nf = oracle_mod.theta_evaluate(x, y, m, 8, TG=1, theta=1e-3, eps2=1e-6)
    assert nf == 0 and nn == 800 * 800
    assert oracle_mod.rel_rms(ax, ay, dax, day) < 1e-13


def test_moments_pyramid_conserves_mass(oracle_mod):
    x, y, m, _, _ = workloads.cluster_mixture(5000, seed=6)
    for G in (1, 7, 16, 19):
        r = oracle_mod.moments(x, y, m, G)
        L = oracle_mod.num_levels(G)
        off, g = 0, G
        for _ in range(L):
            tot = r["mom"][off:off + g * g, 0].sum()
            assert abs(tot - m.sum()) < 1e-9 * m.sum()
            off += g * g
            g = (g + 1) // 2

"""Learned far-field correction in the step.

* A network with all-zero parameters adds nothing: the learned step equals the
  plain step at the same opening angle (relative RMS <= 1e-6).
* Gain: a network trained on pairs from two seeded cluster-mixture systems,
  applied at theta = 0.8 on a third system, lowers the relative RMS force error
  (against the FP64 direct sum on 4,096 targets) below plain theta = 0.8.
* Matched error: the learned step at theta = 0.8 is at least as accurate as a
  plain step at theta <= 0.7 (the largest such plain angle is printed), but not
  as accurate as plain theta = 0.5.  Whether it is faster than the plain step of
  the same accuracy is measured by the benchmark (its learned Pareto).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def accel(sysd, G, theta, mlp=None, theta_lo=0.5, eps=1e-4):
    from barneshut.gb300 import native

    flags = native.BH_FLAG_LEARNED if mlp is not None else 0
    prm = native.make_params(1.0, 1e-5, eps, 0.0, theta, 0, native.BH_PREC_FP32_KAHAN, flags,
                             correction_theta=theta_lo)
    plan = native.Plan([len(sysd[0])], [G], prm)
    if mlp is not None:
        plan.set_correction(mlp)
    plan.load(*sysd)
    plan.create_tree()
    plan.summarize()
    plan.evaluate()
    out = plan.store()
    assert plan.error_flags() == 0
    return plan, out["ax"], out["ay"]


def rel_rms(ax, ay, rx, ry):
    return float(torch.sqrt(((ax - rx) ** 2 + (ay - ry) ** 2).sum() / (rx ** 2 + ry ** 2).sum()))


def test_zero_network_is_plain_step():
    from barneshut.gb300 import learned, workloads

    s = workloads.cluster_mixture(65536, seed=91)
    mlp = learned.LearnedCorrection(params=np.zeros(10448, np.float32))
    _, ax0, ay0 = accel(s, 64, 0.8)
    _, ax1, ay1 = accel(s, 64, 0.8, mlp)
    assert rel_rms(ax1, ay1, ax0, ay0) <= 1e-6


def test_learned_correction_gain():
    from barneshut.gb300 import learned, workloads

    n, G = 262144, 128
    train = [workloads.cluster_mixture(n, seed=101), workloads.cluster_mixture(n, seed=102)]
    mlp, info = learned.train_correction(train, G, 0.8, 0.5, n_pairs=1 << 20, epochs=4)
    assert info["pairs"] > 100000
    # the generated targets carry the analytic quadrupole term the features determine
    assert info["quadrupole_relative_mse"] < 0.9, info
    assert info["relative_mse"] < 0.9, info
    test = workloads.cluster_mixture(n, seed=103)
    t = workloads.precision_subsample(n, 4096, seed=7)
    plan, ax5, ay5 = accel(test, G, 0.5)
    rx, ry = plan.direct_sample(t)
    idx = torch.as_tensor(t, device=ax5.device)
    e05 = rel_rms(ax5[idx], ay5[idx], rx, ry)
    _, ax8, ay8 = accel(test, G, 0.8)
    e08 = rel_rms(ax8[idx], ay8[idx], rx, ry)
    _, axl, ayl = accel(test, G, 0.8, mlp)
    el = rel_rms(axl[idx], ayl[idx], rx, ry)
    # matched error: the largest plain opening angle at least as accurate as the learned step
    plain = {0.5: e05, 0.8: e08}
    for th in (0.6, 0.7):
        _, axp, ayp = accel(test, G, th)
        plain[th] = rel_rms(axp[idx], ayp[idx], rx, ry)
    matched = max([th for th, e in plain.items() if e <= el], default=None)
    print(f"relative RMS force error: plain {', '.join(f'{t} {e:.3e}' for t, e in sorted(plain.items()))}; "
          f"learned 0.8 {el:.3e}, as accurate as plain theta {matched} (training pairs {info['pairs']}, "
          f"rel. MSE {info['relative_mse']:.3f}, quadrupole-only rel. MSE "
          f"{info['quadrupole_relative_mse']:.3f})")
    assert el < 0.9 * e08, (e05, e08, el)
    # the correction at theta 0.8 is worth a plain step at theta <= 0.7, not yet plain 0.5's accuracy
    # (the step-time side of the comparison is the benchmark's learned Pareto)
    assert matched is not None and matched <= 0.7, (plain, el)
    assert el > e05, (e05, el)

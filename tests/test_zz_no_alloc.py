"""bh_direct_sum_noalloc: the direct-sum sampler for callers that cannot
allocate device memory (no plan, no workspace; its scratch is a static device
array inside the library).

Called through the C ABI and checked against the plan-based bh_direct_sample
on the same particles and targets, FP64 relative tolerance 1e-11 (the two
kernels add the same terms in a different order), on two calls in a row: the
second call reuses the static scratch that the first left behind.  This file
is collected last so that a run that stops at its first failure has already
run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _p(t):
    return ctypes.c_void_p(t.data_ptr())


def noalloc(L, x, y, m, targets, gconst, eps):
    n = x.numel()
    t = torch.as_tensor(targets, dtype=torch.int64, device="cuda")
    ax = torch.full((t.numel(),), np.nan, dtype=torch.float64, device="cuda")
    ay = torch.full_like(ax, np.nan)
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = L.bh_direct_sum_noalloc(_p(x), _p(y), _p(m), n, _p(t), t.numel(), gconst, eps, _p(ax),
                                 _p(ay), st)
    assert rc == 0, L.bh_last_error(None)
    return ax.cpu().numpy(), ay.cpu().numpy()


def test_noalloc_matches_direct_sample_twice():
    from barneshut.gb300 import native, workloads

    L = native.load_library()
    n = 20000
    x, y, m, vx, vy = workloads.cluster_mixture(n, seed=123)
    gconst, eps = 1.5, 1e-3
    prm = native.make_params(gconst, 1e-5, eps, 0.0, 0.5)
    plan = native.Plan([n], [16], prm)
    plan.load(x, y, m, vx, vy)  # pid order = the arrays' order
    X, Y, M = (torch.as_tensor(a, device="cuda") for a in (x, y, m))
    rng = np.random.default_rng(5)
    for call in range(2):  # the second call finds the first call's partial sums in scratch
        targets = np.sort(rng.choice(n, size=1000 if call == 0 else 4096, replace=False))
        rx, ry = plan.direct_sample(targets)
        ax, ay = noalloc(L, X, Y, M, targets, gconst, eps)
        np.testing.assert_allclose(ax, rx.cpu().numpy(), rtol=1e-11, atol=0)
        np.testing.assert_allclose(ay, ry.cpu().numpy(), rtol=1e-11, atol=0)


def test_noalloc_rejects_too_many_targets():
    from barneshut.gb300 import native

    L = native.load_library()
    x = torch.zeros(8, dtype=torch.float64, device="cuda")
    t = torch.zeros(native.BH_NOALLOC_MAX_TARGETS + 1, dtype=torch.int64, device="cuda")
    out = torch.zeros(t.numel(), dtype=torch.float64, device="cuda")
    rc = L.bh_direct_sum_noalloc(_p(x), _p(x), _p(x), 8, _p(t), t.numel(), 1.0, 0.0, _p(out),
                                 _p(out), None)
    assert rc == native.BH_ERR_INVALID
    assert b"BH_NOALLOC_MAX_TARGETS" in L.bh_last_error(None)


def test_noalloc_small_n_ragged_targets():
    """Fewer particles (40) than source chunks (64), so most chunks are empty; target indices
    outside [0, n) come back as NaN, as bh_direct_sample reports them; nt = 5 is not a multiple
    of the finishing kernel's block.  Checked against the FP64 oracle's direct sum."""
    from barneshut.gb300 import native, workloads
    from oracle import oracle

    L = native.load_library()
    n = 40
    x, y, m, _, _ = workloads.uniform(n, seed=321)
    X, Y, M = (torch.as_tensor(a, device="cuda") for a in (x, y, m))
    targets = np.array([-1, 0, 39, 40, 17])
    ax, ay = noalloc(L, X, Y, M, targets, 2.0, 1e-2)
    ok = (targets >= 0) & (targets < n)
    assert np.all(np.isnan(ax[~ok])) and np.all(np.isnan(ay[~ok]))
    rx, ry = oracle.direct(x, y, m, gconst=2.0, eps2=1e-4, cutoff=-1.0, targets=targets[ok])
    np.testing.assert_allclose(ax[ok], rx, rtol=1e-11, atol=0)
    np.testing.assert_allclose(ay[ok], ry, rtol=1e-11, atol=0)

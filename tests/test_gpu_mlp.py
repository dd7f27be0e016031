"""tcgen05 MLP kernels (learned far-field correction) against the FP64 NumPy
oracle, which rounds weights and GEMM inputs to BF16 at the same points.

Tolerances: forward outputs relative RMS <= 2e-2 (BF16 activations, FP32
accumulation in a different order); gradients: relative RMS <= 5e-2 per
parameter block and cosine similarity >= 0.998 overall.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


@pytest.fixture(scope="module", autouse=True)
def _gpu():
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def features(n, seed):
    rng = np.random.default_rng(seed)
    u = rng.uniform(-3, 3, size=n)
    v = rng.uniform(-3, 3, size=n)
    q = rng.uniform(0, 0.2, size=(n, 3))
    w = 1.0 / np.sqrt(u * u + v * v + 0.1)
    f = np.zeros((n, 8), dtype=np.float32)
    f[:, 0], f[:, 1], f[:, 2:5], f[:, 5] = u, v, q, w
    return f


def rel_rms(a, b):
    return float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))


def test_forward_matches_oracle():
    from barneshut.gb300.learned import LearnedCorrection
    from oracle import mlp_oracle

    mlp = LearnedCorrection(seed=3)
    f = features(1000, 1)  # not a multiple of the 128-row tile
    out = mlp.forward(torch.from_numpy(f)).cpu().numpy()
    ref, _ = mlp_oracle.forward(mlp.params.cpu().numpy(), f.astype(np.float64))
    assert rel_rms(out, ref) < 2e-2, rel_rms(out, ref)
    mlp.check_errors()


def test_gradient_matches_oracle():
    from barneshut.gb300.learned import LearnedCorrection
    from oracle import mlp_oracle

    mlp = LearnedCorrection(seed=4)
    f = features(777, 2)
    t = np.stack([np.sin(f[:, 0]) * 0.3, np.cos(f[:, 1]) * 0.2], axis=1).astype(np.float32)
    mlp.grad.zero_()
    loss = mlp.grad_batch(torch.from_numpy(f), torch.from_numpy(t))
    g = mlp.grad.cpu().numpy().astype(np.float64)
    ref_loss, rg = mlp_oracle.loss_and_grad(mlp.params.cpu().numpy(), f.astype(np.float64), t)
    assert abs(float(loss.item()) / (777 * 2) - ref_loss) < 2e-2 * ref_loss
    cos = float(np.dot(g, rg) / np.linalg.norm(g) / np.linalg.norm(rg))
    assert cos > 0.998, cos
    for k, (o, s) in mlp_oracle.OFF.items():
        n = int(np.prod(s))
        a, b = g[o:o + n], rg[o:o + n]
        if np.sum(b ** 2) > 0:
            assert rel_rms(a, b) < 5e-2, (k, rel_rms(a, b))
    mlp.check_errors()


def test_training_reduces_loss():
    from barneshut.gb300.learned import LearnedCorrection

    mlp = LearnedCorrection(seed=5)
    f = features(1 << 16, 3)
    t = np.stack([0.3 * np.tanh(f[:, 0]) * f[:, 5], 0.2 * f[:, 2] - 0.1 * f[:, 1] * f[:, 5]],
                 axis=1).astype(np.float32)
    F, T = torch.from_numpy(f).cuda(), torch.from_numpy(t).cuda()
    y0 = mlp.forward(F)
    l0 = float(((y0 - T) ** 2).mean())
    hist = mlp.train(F, T, epochs=3, batch=4096, lr=3e-3)
    y1 = mlp.forward(F)
    l1 = float(((y1 - T) ** 2).mean())
    assert l1 < 0.2 * l0, (l0, l1, hist)

"""Device particle generator (bh_generate) against its CPU restatement (oracle/gen_oracle.py)
and the distributions of the reference's bin/gen_input.py."""
import numpy as np
import pytest

from oracle import gen_oracle


def test_philox_known_answers():
    """Philox4x32-10 known-answer vectors published with the algorithm (Random123)."""
    cases = [((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
             ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
             ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
              (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1))]
    for ctr, key, want in cases:
        got = gen_oracle.philox4x32_10(*[np.array([c], np.uint64) for c in ctr], *key)
        assert tuple(int(v[0]) for v in got) == want


@pytest.mark.parametrize("dist", [gen_oracle.UNIFORM, gen_oracle.GAUSS, gen_oracle.CLUSTER])
def test_oracle_distributions(dist):
    x, y, m, vx, vy = gen_oracle.generate(dist, 200000, seed=12345)
    if dist == gen_oracle.UNIFORM:
        assert x.min() >= 0 and x.max() < 499 and abs(x.mean() - 249.5) < 1.5
        assert abs(np.var(x) - 499 ** 2 / 12) < 0.01 * 499 ** 2 / 12
    elif dist == gen_oracle.GAUSS:
        assert abs(x.mean() - 249.5) < 0.5 and abs(np.std(y) - 499 / 12) < 0.01 * 499 / 12
    else:
        assert x.min() >= 0 and x.max() < 1 and y.max() < 1
        assert np.all((m >= 1) & (m < 2)) and np.all(vx == 0)
    if dist != gen_oracle.CLUSTER:
        assert np.all((m >= 0.5) & (m < 5)) and np.all((vx >= -1) & (vx < 1))
        assert abs(m.mean() - 2.75) < 0.02
    # a pure function of the seed
    x2 = gen_oracle.generate(dist, 1000, seed=12345)[0]
    assert np.array_equal(x2, x[:1000])


@pytest.mark.gpu
@pytest.mark.parametrize("dist", [0, 1, 2])
def test_gpu_generator_matches_oracle(dist):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from barneshut.gb300 import native

    n, seed = 300001, 987654321012345
    out = native.generate(dist, n, seed, device="cuda:0")
    ref = gen_oracle.generate(dist, n, seed)
    for k, r in zip(("x", "y", "m", "vx", "vy"), ref):
        g = out[k].cpu().numpy()
        if dist == 0 or k in ("m", "vx", "vy"):
            np.testing.assert_array_equal(g, r)  # uniform draws: bit-exact
        else:  # Box-Muller: device sincospi/log vs numpy sin/cos/log, and FMA contraction
            np.testing.assert_allclose(g, r, rtol=0, atol=1e-12 * max(1.0, float(np.abs(r).max())))

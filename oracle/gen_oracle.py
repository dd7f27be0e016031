"""CPU restatement of the device particle generator (bh_generate) -- test infrastructure only.

The reference's generator is python-bh/bin/gen_input.py:38-55 (a per-particle host loop over
numpy's default_rng); its distributions are restated on the device with a counter-based
generator, Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1,
2, 3", SC 2011).  This module restates that generator in numpy, vectorised over particles, so
tests can compare the device output bit for bit (uniform draws) or to rounding (Box-Muller
draws, where the device's sincospi/log and numpy's sin/cos/log may differ in the last ulp).
``philox4x32_10`` is pinned by the algorithm's published known-answer vectors in the tests.
"""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint64(0x9E3779B9), np.uint64(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)
UNIFORM, GAUSS, CLUSTER = 0, 1, 2
DOMAIN = 499.0  # gen_input.py: DOMAIN_SIZE - 1


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    """Ten Philox rounds on arrays of 32-bit words (held in uint64); returns four arrays."""
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint64) & MASK for v in (c0, c1, c2, c3))
    k0 = np.uint64(int(k0) & 0xFFFFFFFF)
    k1 = np.uint64(int(k1) & 0xFFFFFFFF)
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & MASK, lo1, (hi0 ^ c3 ^ k1) & MASK, lo0
        k0 = (k0 + W0) & MASK
        k1 = (k1 + W1) & MASK
    return c0, c1, c2, c3


def u53(a, b):
    """Double in [0, 1) from the 27 high bits of a and 26 of b."""
    return ((a >> np.uint64(5)).astype(np.float64) * 67108864.0 +
            (b >> np.uint64(6)).astype(np.float64)) * (1.0 / 9007199254740992.0)


def _box_muller(u, v):
    r = np.sqrt(-2.0 * np.log(1.0 - u))
    return r * np.cos(2.0 * np.pi * v), r * np.sin(2.0 * np.pi * v)


def generate(distribution, n, seed):
    """(x, y, m, vx, vy) as the device generator draws them."""
    i = np.arange(n, dtype=np.uint64)
    ilo, ihi = i & MASK, i >> np.uint64(32)
    k0, k1 = int(seed) & 0xFFFFFFFF, (int(seed) >> 32) & 0xFFFFFFFF
    zero = np.zeros(n, dtype=np.uint64)
    r0 = philox4x32_10(ilo, ihi, zero, zero, k0, k1)
    r1 = philox4x32_10(ilo, ihi, zero + np.uint64(1), zero, k0, k1)
    r2 = philox4x32_10(ilo, ihi, zero + np.uint64(2), zero, k0, k1)
    u0, u1 = u53(r0[0], r0[1]), u53(r0[2], r0[3])
    u2, u3 = u53(r1[0], r1[1]), u53(r1[2], r1[3])
    u4 = u53(r2[0], r2[1])
    if distribution == CLUSTER:
        c = np.minimum((u1 * 8.0).astype(np.int64), 7)
        rc = philox4x32_10(np.arange(8, dtype=np.uint64), np.zeros(8, np.uint64), np.zeros(8, np.uint64),
                           np.ones(8, np.uint64), k0, k1)
        cx = 0.2 + 0.6 * u53(rc[0], rc[1])
        cy = 0.2 + 0.6 * u53(rc[2], rc[3])
        z0, z1 = _box_muller(u2, u3)
        top = 1.0 - 2.0 ** -24
        gx = np.minimum(np.maximum(cx[c] + 0.05 * z0, 0.0), top)
        gy = np.minimum(np.maximum(cy[c] + 0.05 * z1, 0.0), top)
        bg = u0 < 0.2
        x = np.where(bg, u2, gx)
        y = np.where(bg, u3, gy)
        return x, y, 1.0 + u4, np.zeros(n), np.zeros(n)
    if distribution == GAUSS:
        z0, z1 = _box_muller(u0, u1)
        x = 0.5 * DOMAIN + (DOMAIN / 12.0) * z0
        y = 0.5 * DOMAIN + (DOMAIN / 12.0) * z1
    else:
        x, y = u0 * DOMAIN, u1 * DOMAIN
    return x, y, 0.5 + u4 * (5.0 - 0.5), (u2 - 0.5) * 2.0, (u3 - 0.5) * 2.0

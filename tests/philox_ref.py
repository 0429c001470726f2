"""Host restatement of the on-device sampler, for the tests: Philox4x32-10
(Salmon, Moraes, Dror, Shaw, "Parallel random numbers: as easy as 1, 2, 3",
SC'11) in numpy, and the Box-Muller normals the sampler derives from it."""
import numpy as np

M0, M1 = 0xD2511F53, 0xCD9E8D57
W0, W1 = 0x9E3779B9, 0xBB67AE85
MASK = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    """Vectorised Philox4x32-10: ctr (4, n) uint64 holding 32-bit words, key (2,)."""
    x = [np.asarray(c, dtype=np.uint64) & MASK for c in ctr]
    k0, k1 = np.uint64(key[0]), np.uint64(key[1])
    for r in range(10):
        if r > 0:
            k0 = (k0 + np.uint64(W0)) & np.uint64(MASK)
            k1 = (k1 + np.uint64(W1)) & np.uint64(MASK)
        p0 = np.uint64(M0) * x[0]
        p1 = np.uint64(M1) * x[2]
        hi0, lo0 = p0 >> np.uint64(32), p0 & np.uint64(MASK)
        hi1, lo1 = p1 >> np.uint64(32), p1 & np.uint64(MASK)
        x = [hi1 ^ x[1] ^ k0, lo1, hi0 ^ x[3] ^ k1, lo0]
    return x


def normals_host(seed, realization, n_modes):
    j = np.arange(n_modes, dtype=np.uint64)
    key = (seed & MASK, (seed >> 32) & MASK)
    out = []
    for draw in range(3):
        w = philox4x32_10([j & np.uint64(MASK), j >> np.uint64(32),
                           np.full(n_modes, realization & MASK, dtype=np.uint64),
                           np.full(n_modes, draw, dtype=np.uint64)], key)
        u = lambda hi, lo: (((hi >> np.uint64(5)) << np.uint64(26)) | (lo >> np.uint64(6))).astype(
            np.float64) * 2.0 ** -53
        u1 = 1.0 - u(w[0], w[1])
        u2 = u(w[2], w[3])
        r = np.sqrt(-2.0 * np.log(u1))
        s, c = sincospi(2.0 * u2)
        out += [r * c, r * s]
    return out


def sincospi(x):
    """sin(pi x), cos(pi x) to about one ulp of the result, also near their
    zeros: exact reductions to |w| <= 1/4 before np.sin / np.cos of pi w."""
    x = np.asarray(x, dtype=np.float64)
    y = x - 2.0 * np.rint(x / 2.0)                    # [-1, 1], exact
    flip = np.abs(y) > 0.5
    z = np.where(flip, np.sign(y) - y, y)             # [-1/2, 1/2], exact
    # sin(pi y) = sin(pi z); cos(pi y) = -cos(pi z) where flipped
    far = np.abs(z) > 0.25
    w = np.where(far, 0.5 - np.abs(z), z)             # exact
    sw, cw = np.sin(np.pi * w), np.cos(np.pi * w)
    s = np.where(far, np.sign(z) * cw, sw)
    c = np.where(far, sw, cw)
    return s, np.where(flip, -c, c)

"""NumPy statement of the in-kernel Wiener generator (test infrastructure).

Particles are taken in pairs (2p, 2p+1).  Philox-4x32-10 (Salmon et al.,
SC'11) on the counter (step low word, step high word, p, 0x5d12) with the
member seed as key gives four words; their top 21 bits make four uniforms
and their low 11 bits, joined two words at a time, two 22-bit uniforms
(u = (x + 1/2) 2^-b).  Three Box-Muller pairs (radius sqrt(-2 ln u), angle
2 pi u - pi): words 0, 1 -> components 0, 1 of particle 2p; words 2, 3 ->
components 0, 1 of 2p+1; the two low parts -> component 2 of 2p (cosine)
and of 2p+1 (sine).  The integer part is exact; the device's float32
log/sqrt/sin/cos differ from these by far less than the tests' tolerance.
"""
import numpy as np

M0, M1 = np.uint64(0xD2511F53), np.uint64(0xCD9E8D57)
W0, W1 = np.uint32(0x9E3779B9), np.uint32(0xBB67AE85)
MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c0, c1, c2, c3 = (np.asarray(v, dtype=np.uint64) for v in (c0, c1, c2, c3))
    k0 = np.uint64(k0)
    k1 = np.uint64(k1)
    for _ in range(10):
        p0 = M0 * c0
        p1 = M1 * c2
        hi0, lo0 = p0 >> np.uint64(32), p0 & MASK
        hi1, lo1 = p1 >> np.uint64(32), p1 & MASK
        c0, c1, c2, c3 = (hi1 ^ c1 ^ k0) & MASK, lo1, (hi0 ^ c3 ^ k1) & MASK, lo0
        k0 = (k0 + np.uint64(W0)) & MASK
        k1 = (k1 + np.uint64(W1)) & MASK
    return [v.astype(np.uint32) for v in (c0, c1, c2, c3)]


def u21(w):
    return (np.float32(w >> np.uint32(11)) * np.float32(2.0 ** -21)
            + np.float32(2.0 ** -22)).astype(np.float32)


def u22(x):
    return (np.float32(x) * np.float32(2.0 ** -22) + np.float32(2.0 ** -23)).astype(np.float32)


def low22(a, b):
    return ((a & np.uint32(0x7FF)) << np.uint32(11)) | (b & np.uint32(0x7FF))


def _box_muller(ur, ut):
    r = np.sqrt(-2.0 * np.log(ur.astype(np.float64)))
    twopi, pi = np.float64(np.float32(2 * np.pi)), np.float64(np.float32(np.pi))
    # fused multiply-add: exact product, one rounding
    a = (twopi * ut.astype(np.float64) - pi).astype(np.float32).astype(np.float64)
    return r * np.cos(a), r * np.sin(a)


def wiener(seed, n_particles, n_steps):
    """[n_steps][3n] increments, as magpy_wiener_increments returns them."""
    k = np.arange(1, n_steps + 1, dtype=np.uint64)[:, None]
    q = np.arange(n_particles, dtype=np.uint64)[None, :]
    k, q = np.broadcast_arrays(k, q)
    r = philox4x32_10(k & MASK, k >> np.uint64(32), q >> np.uint64(1),
                      np.full_like(q, 0x5D12), seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    odd = (q & np.uint64(1)) == 1
    n0, n1 = _box_muller(u21(np.where(odd, r[2], r[0])), u21(np.where(odd, r[3], r[1])))
    c0, c1 = _box_muller(u22(low22(r[0], r[1])), u22(low22(r[2], r[3])))
    out = np.stack([n0, n1, np.where(odd, c1, c0)], axis=-1)
    return out.reshape(n_steps, 3 * n_particles).astype(np.float32).astype(np.float64)

"""NumPy statement of the in-kernel Wiener generator (test infrastructure).

Philox-4x32-10 (Salmon et al., SC'11) on the counter (step low word, step high
word, particle, 0x5d11) with the member seed as key, then Box-Muller on the
top 24 bits of each word (angle uniform on (-pi, pi)).  The integer part is exact; the float32
log/sqrt/sin/cos differ from the device's by a few ulp.
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


def u24(x):
    return (np.float32(x >> np.uint32(8)) * np.float32(5.9604644775390625e-8)
            + np.float32(2.98023223876953125e-8)).astype(np.float32)


def wiener(seed, n_particles, n_steps):
    """[n_steps][3n] increments, as magpy_wiener_increments returns them."""
    k = np.arange(1, n_steps + 1, dtype=np.uint64)[:, None]
    q = np.arange(n_particles, dtype=np.uint64)[None, :]
    k, q = np.broadcast_arrays(k, q)
    r = philox4x32_10(k & MASK, k >> np.uint64(32), q, np.full_like(q, 0x5D11),
                      seed & 0xFFFFFFFF, (seed >> 32) & 0xFFFFFFFF)
    r0 = np.sqrt(np.float32(-2.0) * np.log(u24(r[0])))
    r1 = np.sqrt(np.float32(-2.0) * np.log(u24(r[2])))
    twopi, pi = np.float64(np.float32(2 * np.pi)), np.float64(np.float32(np.pi))
    # fused multiply-add: exact product, one rounding
    a0 = (twopi * u24(r[1]).astype(np.float64) - pi).astype(np.float32)
    a1 = (twopi * u24(r[3]).astype(np.float64) - pi).astype(np.float32)
    out = np.stack([r0 * np.cos(a0), r0 * np.sin(a0), r1 * np.cos(a1)], axis=-1)
    return out.reshape(n_steps, 3 * n_particles).astype(np.float64)

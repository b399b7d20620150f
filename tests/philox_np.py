"""Vectorised Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11) in numpy.

Test-side generator of the engine's counter-based uniforms: point i, dimension
block b, stream id s -> counter (i lo, i hi, b, s), key (seed lo, seed hi); each
block yields two 53-bit doubles in [0, 1).
"""
import numpy as np

_M0 = np.uint64(0xD2511F53)
_M1 = np.uint64(0xCD9E8D57)
_W0 = np.uint32(0x9E3779B9)
_W1 = np.uint32(0xBB67AE85)
_MASK = np.uint64(0xFFFFFFFF)


def philox4x32_10(c0, c1, c2, c3, k0, k1):
    c = [np.asarray(x, dtype=np.uint32).copy() for x in (c0, c1, c2, c3)]
    k0 = np.uint32(k0)
    k1 = np.uint32(k1)
    with np.errstate(over="ignore"):
        for r in range(10):
            p0 = _M0 * c[0].astype(np.uint64)
            p1 = _M1 * c[2].astype(np.uint64)
            hi0 = (p0 >> np.uint64(32)).astype(np.uint32)
            lo0 = (p0 & _MASK).astype(np.uint32)
            hi1 = (p1 >> np.uint64(32)).astype(np.uint32)
            lo1 = (p1 & _MASK).astype(np.uint32)
            c = [hi1 ^ c[1] ^ k0, lo1, hi0 ^ c[3] ^ k1, lo0]
            if r < 9:
                k0 = np.uint32(k0 + _W0)
                k1 = np.uint32(k1 + _W1)
    return c


def uniforms(seed, n, dim, first=0, stream=0):
    """(n, dim) float64 uniforms of points first .. first + n - 1."""
    idx = np.arange(first, first + n, dtype=np.uint64)
    lo = (idx & _MASK).astype(np.uint32)
    hi = (idx >> np.uint64(32)).astype(np.uint32)
    out = np.empty((n, dim), dtype=np.float64)
    k0 = np.uint32(seed & 0xFFFFFFFF)
    k1 = np.uint32((seed >> 32) & 0xFFFFFFFF)
    for blk in range((dim + 1) // 2):
        o = philox4x32_10(lo, hi, np.full(n, blk, np.uint32), np.full(n, stream, np.uint32), k0, k1)
        a = (o[1].astype(np.uint64) << np.uint64(32)) | o[0].astype(np.uint64)
        b = (o[3].astype(np.uint64) << np.uint64(32)) | o[2].astype(np.uint64)
        out[:, 2 * blk] = (a >> np.uint64(11)).astype(np.float64) * 2.0**-53
        if 2 * blk + 1 < dim:
            out[:, 2 * blk + 1] = (b >> np.uint64(11)).astype(np.float64) * 2.0**-53
    return out

"""ctypes access to the CPU oracle (oracle/_build/liborc.so).

TEST INFRASTRUCTURE: imported only by tests/, __graft_entry__.smoke() and the CPU
legs of bench.py, as the checker / CPU baseline. Never on the product path.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(_HERE, "_build", "liborc.so")
LIB_LD = os.path.join(_HERE, "_build", "liborc_ld.so")  # the same restatement in long double
_lib = None
_lib_ld = None


def build():
    subprocess.check_call(["make", "-s", "-C", _HERE])


def lib(long_double=False):
    """The oracle library; long_double selects the extended-precision build (same code and
    constants, long double arithmetic: 64-bit significand on x86, 113-bit on aarch64)."""
    global _lib, _lib_ld
    if long_double and _lib_ld is not None:
        return _lib_ld
    if not long_double and _lib is not None:
        return _lib
    path = LIB_LD if long_double else LIB
    if True:
        if not os.path.exists(path):
            build()
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.orc_weights.restype = ctypes.c_int
        L.orc_weights.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int32, vp, vp, vp, vp,
                                  ctypes.c_int32, ctypes.c_int32]
        L.orc_eikonal.restype = ctypes.c_int
        L.orc_eikonal.argtypes = [vp, ctypes.c_int32, ctypes.c_int32, vp, vp, vp, ctypes.c_int32]
        L.orc_observables.restype = ctypes.c_int
        L.orc_observables.argtypes = [vp, vp, ctypes.c_int64, ctypes.c_int32, vp, vp,
                                      ctypes.c_int32]
        L.orc_bessel_j0.restype = ctypes.c_double
        L.orc_bessel_j0.argtypes = [ctypes.c_double]
        L.orc_vegas_grid_init.argtypes = [ctypes.c_int32, ctypes.c_int32, vp]
        L.orc_vegas_refine.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_double, vp, vp]
        L.orc_vegas_map.argtypes = [ctypes.c_int32, ctypes.c_int32, vp, vp, ctypes.c_int64, vp, vp,
                                    vp]
        L.orc_uniforms.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_int64,
                                   ctypes.c_int64, ctypes.c_int32, vp]
        if long_double:
            _lib_ld = L
        else:
            _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def weights(params, u, msa=None, nthreads=1, with_rec=False, long_double=False):
    """(w, flags[, rec]) for u of shape (n, dim) (8 for 2-body states, 12 or 14 for two-body
    cascades, 14 for 4-body states). rec per point: t1, t2, m2, the 4-momenta (px, py, pz, E)
    of pfinal[1..4] and of the four cascade daughters. long_double: evaluate in the extended-
    precision build (results rounded to double)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    n, dim = u.shape
    w = np.zeros(n)
    fl = np.zeros(n, dtype=np.uint8)
    rec = np.zeros((n, 35)) if with_rec else None
    n_kt2 = 0
    if msa is not None:
        msa = np.ascontiguousarray(msa, dtype=np.float64)
        n_kt2 = msa.shape[0] - 1
    st = lib(long_double).orc_weights(ctypes.byref(params), _p(u), n, dim, _p(w), _p(fl),
                                      _p(rec), _p(msa), n_kt2, nthreads)
    if st != 0:
        raise RuntimeError("orc_weights status %d" % st)
    return (w, fl, rec) if with_rec else (w, fl)


def observables(params, u, nthreads=4):
    """(obs (n, 20), ok (n,)): the histogram observables (GRN_OBS_* order) of each point that
    passes the kinematics."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    n, dim = u.shape
    obs = np.full((n, 20), np.nan)
    ok = np.zeros(n, dtype=np.uint8)
    st = lib().orc_observables(ctypes.byref(params), _p(u), n, dim, _p(obs), _p(ok), nthreads)
    if st != 0:
        raise RuntimeError("orc_observables status %d" % st)
    return obs, ok.astype(bool)


def eikonal(params, n_bt, n_kt2, nthreads=8, with_msa=True):
    mbt = np.zeros((n_bt + 1, 3))
    msa = np.zeros((n_kt2 + 1, 3)) if with_msa else None
    xs = np.zeros(3)
    st = lib().orc_eikonal(ctypes.byref(params), n_bt, n_kt2, _p(mbt), _p(msa), _p(xs), nthreads)
    if st != 0:
        raise RuntimeError("orc_eikonal status %d" % st)
    return mbt, msa, xs


def bessel_j0(x):
    return lib().orc_bessel_j0(float(x))


def vegas_grid_init(bins, dim):
    x = np.zeros((bins, dim))
    lib().orc_vegas_grid_init(bins, dim, _p(x))
    return x


def vegas_refine(xmat, f2mat, lam=1.5):
    xmat = np.ascontiguousarray(xmat, dtype=np.float64).copy()
    f2 = np.ascontiguousarray(f2mat, dtype=np.float64).copy()
    bins, dim = xmat.shape
    lib().orc_vegas_refine(bins, dim, lam, _p(xmat), _p(f2))
    return xmat


def vegas_map(xmat, r):
    xmat = np.ascontiguousarray(xmat, dtype=np.float64)
    r = np.ascontiguousarray(r, dtype=np.float64)
    bins, dim = xmat.shape
    n = r.shape[0]
    x = np.zeros_like(r)
    vw = np.zeros(n)
    b = np.zeros((n, dim), dtype=np.int32)
    lib().orc_vegas_map(bins, dim, _p(xmat), _p(r), n, _p(x), _p(vw), _p(b))
    return x, vw, b


def uniforms(seed, n, dim, first=0, stream=0):
    out = np.zeros((n, dim))
    lib().orc_uniforms(seed, stream, first, n, dim, _p(out))
    return out

"""grn_event_weights_noalloc: the allocation-free variant of grn_event_weights.

It exists for callers that may not allocate device memory while they run (their
device memory belongs to their own pool allocator, or was sized once at start-up and
must not meet an out-of-memory error or cudaFree's synchronisation mid-run). Its
scratch (the screened work list) is a fixed array inside the library. This test
calls it through the C ABI on device buffers and checks it against grn_event_weights
on two calls in a row (the shared scratch keeps the previous call's contents).
Collected last on purpose (file name), and independent of the other tests.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_FP64 = 5e-10   # the FP64 parity tolerance of the other GPU tests
TOL_MIXED = 1e-5   # the FP32-loop tolerance of the other GPU tests


def _engine(params_screened):
    import graniitti_gb300 as g
    P = params_screened
    P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = 15, 12, 1.75
    e = g.Engine(P, 0)
    e.eikonal_build(200, 2000)
    return e


def _call_noalloc(e, u, w, f, prec):
    return e.lib.grn_event_weights_noalloc(e.h, ctypes.c_void_p(u.data_ptr()), u.shape[0],
                                           e.dim, ctypes.c_void_p(w.data_ptr()),
                                           ctypes.c_void_p(f.data_ptr()), prec)


def _close(a, b, tol):
    nz = b > 0
    assert np.array_equal(a > 0, nz)
    return np.all(np.abs(a[nz] - b[nz]) <= tol * b[nz])


def test_noalloc_matches_event_weights_twice(gpu, params_screened):
    import torch
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi
    e = _engine(params_screened)
    for call, (seed, n) in enumerate(((21, 3000), (22, 1777))):
        uh = e.uniforms(seed=seed, n=n)
        u = torch.from_numpy(uh).cuda()
        for prec, tol in ((g.FP64, TOL_FP64), (g.MIXED, TOL_MIXED)):
            w = torch.zeros(n, dtype=torch.float64, device="cuda")
            f = torch.zeros(n, dtype=torch.uint8, device="cuda")
            st = _call_noalloc(e, u, w, f, prec)
            assert st == _abi.GRN_OK, e.lib.grn_last_error()
            torch.cuda.synchronize()
            w_ref, f_ref = e.event_weights(uh, prec=prec)
            assert np.array_equal(f.cpu().numpy(), f_ref), "call %d prec %d flags" % (call, prec)
            assert _close(w.cpu().numpy(), w_ref, tol), "call %d prec %d weights" % (call, prec)
            assert (w_ref > 0).sum() > n // 2


def test_noalloc_14_dimensional_cascade(gpu):
    """The scratch serves 14-dimensional points too: the screened tensor-pomeron
    rho rho -> pi+ pi- pi+ pi- cascade (generic loop in both entry points, so MIXED
    agrees to the FP64 tolerance as well), two calls in a row."""
    import os
    import torch
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi, card
    from conftest import GOLDEN
    P = card.build_params(card.read_card(os.path.join(GOLDEN, "cards", "pp_con_pipi_screened.json")),
                          "PP[CONTENSOR]<F> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}")
    P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = 15, 12, 1.75
    e = g.Engine(P, 0)
    assert e.dim == 14
    e.eikonal_build(200, 2000)
    for call, (seed, n) in enumerate(((31, 1500), (32, 777))):
        uh = e.uniforms(seed=seed, n=n)
        u = torch.from_numpy(uh).cuda()
        for prec in (g.FP64, g.MIXED):
            w = torch.zeros(n, dtype=torch.float64, device="cuda")
            f = torch.zeros(n, dtype=torch.uint8, device="cuda")
            st = _call_noalloc(e, u, w, f, prec)
            assert st == _abi.GRN_OK, e.lib.grn_last_error()
            torch.cuda.synchronize()
            w_ref, f_ref = e.event_weights(uh, prec=prec)
            assert np.array_equal(f.cpu().numpy(), f_ref), "call %d prec %d flags" % (call, prec)
            assert _close(w.cpu().numpy(), w_ref, TOL_FP64), "call %d prec %d" % (call, prec)
            assert (w_ref > 0).sum() > 0
    # a dimension other than the engine's is refused with the engine's dimension named
    st = e.lib.grn_event_weights_noalloc(e.h, ctypes.c_void_p(u.data_ptr()), 4, 8,
                                         ctypes.c_void_p(w.data_ptr()), None, 0)
    assert st == _abi.GRN_ERR_INVALID and b"grn_dim() = 14" in e.lib.grn_last_error()
    e.close()


def test_noalloc_rejects_oversize_and_host_buffers(gpu, params_screened):
    import torch
    from graniitti_gb300 import _abi
    e = _engine(params_screened)
    u = torch.zeros((4, 8), dtype=torch.float64, device="cuda")
    w = torch.zeros(4, dtype=torch.float64, device="cuda")
    f = torch.zeros(4, dtype=torch.uint8, device="cuda")
    st = e.lib.grn_event_weights_noalloc(e.h, ctypes.c_void_p(u.data_ptr()),
                                         _abi.GRN_NOALLOC_MAX_POINTS + 1, 8,
                                         ctypes.c_void_p(w.data_ptr()),
                                         ctypes.c_void_p(f.data_ptr()), 0)
    assert st == _abi.GRN_ERR_INVALID and b"GRN_NOALLOC_MAX_POINTS" in e.lib.grn_last_error()
    uh = np.full((4, 8), 0.5)
    wh = np.zeros(4)
    st = e.lib.grn_event_weights_noalloc(e.h, uh.ctypes.data_as(ctypes.c_void_p), 4, 8,
                                         wh.ctypes.data_as(ctypes.c_void_p), None, 0)
    assert st == _abi.GRN_ERR_INVALID and b"device pointers" in e.lib.grn_last_error()

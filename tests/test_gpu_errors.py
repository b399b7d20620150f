"""Error behaviour at the C ABI (status codes, no exceptions, no device faults)."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_status_codes(gpu, params, params_screened):
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi
    lib = _abi.load_library()
    bad = _abi.ProcessParams()
    ctypes.memmove(ctypes.byref(bad), ctypes.byref(params), ctypes.sizeof(bad))
    bad.n_central = 3  # 2- and 4-body central states are built
    h = ctypes.c_void_p()
    assert lib.grn_create(ctypes.byref(bad), 0, ctypes.byref(h)) == _abi.GRN_ERR_UNSUPPORTED
    bad.n_central = 2
    bad.regge.offshellFF = 7
    assert lib.grn_create(ctypes.byref(bad), 0, ctypes.byref(h)) == _abi.GRN_ERR_INVALID
    assert b"offshellFF" in lib.grn_last_error()
    # screening without tables
    e = g.Engine(params_screened, 0)
    with pytest.raises(_abi.GrnError) as ex:
        e.event_weights(np.full((4, 8), 0.5))
    assert ex.value.status == _abi.GRN_ERR_STATE
    # loop grid not a multiple of 3
    P = params_screened
    P.loop.n_kt = 16
    e2 = g.Engine(P, 0)
    with pytest.raises(_abi.GrnError):
        e2.eikonal_build(100, 1000)
    P.loop.n_kt = 15
    # dimension mismatch
    e3 = g.Engine(params, 0)
    w = np.zeros(4)
    st = lib.grn_event_weights(e3.h, np.zeros((4, 6)).ctypes.data_as(ctypes.c_void_p), 4, 6,
                               w.ctypes.data_as(ctypes.c_void_p), None, 0)
    assert st == _abi.GRN_ERR_INVALID
    # unweight before any VEGAS pass
    assert lib.grn_unweight(e3.h, 1.0, 1, None, None, None, 0) == _abi.GRN_ERR_STATE


def test_nan_weights_are_zeroed_and_flagged(gpu, params):
    """Non-finite weights (here: NaN inputs) come back as 0 with amplitude_ok off
    (MProcess::CheckInfNan, include/Graniitti/MProcess.h:317-340)."""
    import graniitti_gb300 as g
    e = g.Engine(params, 0)
    u = np.full((8, 8), 0.4)
    u[0, 0] = np.nan
    w, fl = e.event_weights(u)
    assert np.all(np.isfinite(w)) and w[0] == 0.0


def test_flow_wait_timeout_reports_and_recovers(gpu, params):
    """The bounded waits of the tensor-core flow kernel: with the first wait's poll limit set
    to 0 it gives up while the weight copy is in flight; the kernel drains the copy, frees its
    tensor memory and sets its error flag, the call fails with GRN_ERR_CUDA, and the next call
    (default limit) gives the same result as before."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi
    e = g.Engine(params, 0)
    f = g.Flow(e, seed=3)
    rng = np.random.default_rng(1)
    x = rng.random((8, 4096)).astype(np.float32)
    z0, lq0 = f.density(x)
    f.set_wait_polls(0)
    with pytest.raises(_abi.GrnError) as ei:
        f.density(x)
    assert ei.value.status == _abi.GRN_ERR_CUDA and "bounded wait" in str(ei.value)
    f.set_wait_polls(-1)
    z1, lq1 = f.density(x)
    assert np.array_equal(z0, z1) and np.array_equal(lq0, lq1)
    f.close()
    e.close()

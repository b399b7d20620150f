"""Tensor-pomeron resonances (PP[RESTENSOR], MTensorPomeron::ME3) on the GPU through the C ABI:
FP64 weights against the reference's golden vectors and the CPU oracle, the FP32 kt-loop
against FP64, the cross section against the reference's VEGAS, and parameter validation."""
import ctypes
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle_api as orc
from test_gpu_parity import _mixed_ok

pytestmark = pytest.mark.gpu

# The tensor amplitude has zeros in the decay angle where the reference's Cartesian
# contractions lose relative precision (a few points at 1e-9, median 2e-11); the GPU's
# light-cone contraction is the more accurate of the two.
RES_TOL = 5e-9
# Regge resonances: near a zero of the d-wave decay distribution the quadratic form
# f rho_rot f^+ of the spin factor is a small difference of O(1) terms, summed in another
# order on the GPU than in the reference (one point at 9e-9; medians 1e-11 to 2e-11).
REGGE_TOL = 2e-8


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _params(g):
    from graniitti_gb300 import card
    return card.build_params(card.read_card(os.path.join(GOLDEN, "cards", str(g["card"]))),
                             str(g["proc"]))


def _engine(P):
    import graniitti_gb300 as g
    return g.Engine(P, 0)


def _rel(w, wr):
    nz = wr > 0
    assert np.array_equal(w > 0, nz)
    return np.abs(w[nz] - wr[nz]) / wr[nz]


@pytest.mark.parametrize("name", ["rf_tree_weights.npz", "rf_mix_tree_weights.npz",
                                  "rf_kk_tree_weights.npz", "rc_tree_weights.npz",
                                  "rf_f2_1525_tree_weights.npz"] +
                         ["rf_s%d_tree_weights.npz" % j for j in range(1, 7)] +
                         ["rcf_tree_weights.npz", "rcc_tree_weights.npz", "rck_tree_weights.npz"] +
                         ["gr_tree_weights.npz", "grc_tree_weights.npz", "grc_hx_tree_weights.npz",
                          "grc_cm_jz_tree_weights.npz", "grc_nogen_tree_weights.npz",
                          "grc_kk_tree_weights.npz", "grc_c_tree_weights.npz"])
def test_resonance_tree_vs_reference(gpu, name):
    import graniitti_gb300 as g
    gl = _load(name)
    P = _params(gl)
    e = _engine(P)
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    wo, flo = orc.weights(P, gl["u"])
    assert np.array_equal(fl, flo) and np.array_equal(fl & 1, gl["kin"])
    kin = gl["kin"] == 1
    assert np.array_equal(((fl >> 1) & 1)[kin], gl["fid"][kin])
    r = _rel(w, gl["w"])
    print("%s: GPU vs reference max rel %.2e, median %.2e" % (name, r.max(), np.median(r)))
    tol = REGGE_TOL if name.startswith("gr") else RES_TOL
    assert r.max() < tol and np.median(r) < 1e-10
    assert _rel(w, wo).max() < tol
    # tree-level weights do not depend on the loop precision
    wm, _ = e.event_weights(gl["u"], prec=g.MIXED)
    assert np.array_equal(wm, w)


@pytest.mark.parametrize("name", ["rf_screened_15x12_weights.npz",
                                  "rcf_screened_15x12_weights.npz",
                                  "grc_screened_15x12_weights.npz"])
def test_resonance_screened_vs_reference(gpu, name):
    import graniitti_gb300 as g
    gl = _load(name)
    t = _load("eikonal_nbt1024_nkt10000.npz")
    P = _params(gl)
    assert P.screening == 1
    e = _engine(P)
    e.eikonal_set(t["mbt"], t["msa"])
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    assert np.array_equal(fl & 1, gl["kin"])
    r = _rel(w, gl["w"])
    print("screened resonances: GPU FP64 vs reference max rel %.2e" % r.max())
    assert r.max() < RES_TOL
    wm, _ = e.event_weights(gl["u"], prec=g.MIXED)
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = _engine(Pb).event_weights(gl["u"], prec=g.FP64)
    ok, rel = _mixed_ok(wm, w, wb)
    print("screened resonances: mixed vs fp64 max rel %.3e" % rel.max())
    assert ok, rel.max()
    # screening suppresses the resonance on average
    nz = wb > 0
    assert np.sum(w[nz]) < np.sum(wb[nz])


def test_resonance_mixed_loop_vs_fp64_many_points(gpu):
    """FP32 kt-loop of the resonance amplitude against the FP64 loop on 4096 points of the
    screened f0(980) + f2(1270) process (tables built on the device)."""
    import graniitti_gb300 as g
    import philox_np
    gl = _load("rf_screened_15x12_weights.npz")
    P = _params(gl)
    e = _engine(P)
    e.eikonal_build()
    u = philox_np.uniforms(66, 4096, 8)
    w64, fl = e.event_weights(u, prec=g.FP64)
    wm, flm = e.event_weights(u, prec=g.MIXED)
    assert np.array_equal(fl, flm)
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = _engine(Pb).event_weights(u, prec=g.FP64)
    ok, rel = _mixed_ok(wm, w64, wb)
    print("resonance mixed vs fp64 (4096 points): max rel %.3e, median %.3e" %
          (rel.max(), np.median(rel)))
    assert ok, rel.max()


@pytest.mark.parametrize("name", ["rf_vegas_sigma.json", "grc_vegas_sigma.json"])
def test_resonance_cross_section_vs_reference_vegas(gpu, name):
    """Integrated cross sections against the reference's own VEGAS runs: tensor-pomeron
    f2(1270) -> pi+ pi-, and the Regge f0(980) + f2(1270) + continuum -> pi+ pi-."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi, card
    ref = json.load(open(os.path.join(GOLDEN, name)))
    P = card.build_params(card.read_card(os.path.join(GOLDEN, "cards", ref["card"])),
                          ref["process"])
    e = g.Engine(P, 0)
    vp = _abi.VegasParams()
    vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 8, 1 << 21, 1.5
    vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 2e-4, 3, 0, 21
    r = e.vegas_integrate(vp)
    pull = (r.sigma - ref["sigma_barn"]) / np.hypot(r.sigma_err, ref["sigma_err_barn"])
    print("sigma %s: GPU %.5e +- %.1e, reference %.5e +- %.1e, pull %.2f" %
          (ref["process"], r.sigma, r.sigma_err, ref["sigma_barn"], ref["sigma_err_barn"], pull))
    assert abs(pull) < 4


def test_resonance_parameter_validation(gpu):
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi
    gl = _load("rf_tree_weights.npz")
    P = _params(gl)
    lib = _abi.load_library()

    def status(mod):
        Q = type(P)()
        ctypes.memmove(ctypes.byref(Q), ctypes.byref(P), ctypes.sizeof(P))
        mod(Q)
        h = ctypes.c_void_p()
        st = lib.grn_create(ctypes.byref(Q), 0, ctypes.byref(h))
        if h.value:
            lib.grn_destroy(h)
        return st

    assert status(lambda Q: None) == _abi.GRN_OK
    assert status(lambda Q: setattr(Q, "n_res", 0)) == _abi.GRN_ERR_INVALID
    assert status(lambda Q: setattr(Q, "n_res", 5)) == _abi.GRN_ERR_INVALID
    assert status(lambda Q: Q.res[0].g_tensor.__setitem__(1, 0.5)) == _abi.GRN_OK
    assert status(lambda Q: (setattr(Q.res[0], "J", 0), Q.res[0].g_tensor.__setitem__(2, 0.5))) \
        == _abi.GRN_ERR_UNSUPPORTED
    assert status(lambda Q: setattr(Q.res[0], "J", 1)) == _abi.GRN_ERR_UNSUPPORTED
    assert status(lambda Q: setattr(Q.res[0], "M", -1.0)) == _abi.GRN_ERR_INVALID
    assert status(lambda Q: Q.m_central.__setitem__(1, 0.2)) == _abi.GRN_ERR_UNSUPPORTED


@pytest.mark.parametrize("g", ["g0:0, g1:1", "g0:0, g2:1", "g0:0, g3:1", "g0:0, g4:1",
                               "g0:0, g5:1", "g0:0, g6:1", "g0:2, g1:1, g4:0.5"])
def test_tensor_structures_mixed_loop_vs_fp64(gpu, g):
    """FP32 kt-loop of each J = 2 coupling structure against the FP64 loop, 4096 points
    (events whose FP32 error estimate exceeds 1e-5 are redone in FP64)."""
    import graniitti_gb300 as gg
    import philox_np
    from graniitti_gb300 import card
    c = card.read_card(os.path.join(GOLDEN, "cards", "pp_res_pipi_screened.json"))
    P = card.build_params(c, "PP[RESTENSOR]<F> -> pi+ pi- @R[f2_1270]{%s}" % g)
    e = _engine(P)
    e.eikonal_build()
    u = philox_np.uniforms(67, 4096, 8)
    w64, fl = e.event_weights(u, prec=gg.FP64)
    wm, flm = e.event_weights(u, prec=gg.MIXED)
    assert np.array_equal(fl, flm)
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = _engine(Pb).event_weights(u, prec=gg.FP64)
    ok, rel = _mixed_ok(wm, w64, wb)
    print("structures {%s}: mixed vs fp64 max rel %.3e, median %.3e" %
          (g, rel.max(), np.median(rel)))
    assert ok, rel.max()


def _structure1_engine():
    from graniitti_gb300 import card
    c = card.read_card(os.path.join(GOLDEN, "cards", "pp_res_pipi_screened.json"))
    P = card.build_params(c, "PP[RESTENSOR]<F> -> pi+ pi- @R[f2_1270]{g0:0, g1:1}")
    e = _engine(P)
    e.eikonal_build()
    return P, e


def test_fp32_loop_refinement_structure1(gpu):
    """Structure 1 ((l,s) = (2,0) - (2,2)) at small forward pT: its phi-rings cancel by up to
    10^12, so the plain FP32 loop is wrong by orders of magnitude on many events; the error
    estimate sends those to the FP64 loop and the mixed weights meet the FP64 ones."""
    import graniitti_gb300 as gg
    import philox_np
    P, e = _structure1_engine()
    u = philox_np.uniforms(67, 4096, 8)
    w64, _ = e.event_weights(u, prec=gg.FP64)
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = _engine(Pb).event_weights(u, prec=gg.FP64)
    e.set_tuning(fp64_refine=0)
    assert e.tuning().fp64_refine == 0
    w32, _ = e.event_weights(u, prec=gg.MIXED)
    ok32, rel32 = _mixed_ok(w32, w64, wb)
    e.set_tuning(fp64_refine=1)
    wm, _ = e.event_weights(u, prec=gg.MIXED)
    ok, rel = _mixed_ok(wm, w64, wb)
    print("structure 1: plain FP32 loop max rel %.2e (median %.2e); refined %.2e" %
          (rel32.max(), np.median(rel32), rel.max()))
    assert not ok32 and rel32.max() > 1e-2
    assert ok, rel.max()


def test_fp32_loop_refinement_vegas_pass(gpu):
    """A VEGAS pass of structure 1 on the mixed loop reports the refined events and gives
    the FP64 pass's integral on the same points."""
    import graniitti_gb300 as gg
    from graniitti_gb300 import _abi
    res = {}
    for prec in (gg.FP64, gg.MIXED):
        _, e = _structure1_engine()
        vp = _abi.VegasParams()
        vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, 1 << 16, 1.5
        vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, prec, 5
        e.vegas_init(vp)
        res[prec] = e.vegas_iteration(mode=1, refine=False, iter_id=3)
        e.close()
    r64, rm = res[gg.FP64], res[gg.MIXED]
    print("structure 1 VEGAS pass: %d of %d screened events refined; I mixed %.8e, FP64 %.8e"
          % (rm.refined, int(rm.fidcuts_ok), rm.I_this, r64.I_this))
    assert r64.refined == 0 and 0 < rm.refined <= rm.fidcuts_ok
    assert rm.I_this == pytest.approx(r64.I_this, rel=1e-5)
    assert rm.maxf == pytest.approx(r64.maxf, rel=1e-5)
    assert rm.nan_count == r64.nan_count


def test_far_off_shell_events_without_refinement():
    """f2(1270) alone on the 63 x 33 grid with the FP64 refinement off: events ~3 GeV off the
    pole, whose resonance factors are FP64-subnormal, keep a finite FP32 loop (the event scale
    stays finite), so a VEGAS pass meets no NaN weight and gives the refined pass's integral."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi, card
    from conftest import CARD_SCR
    c = card.read_card(CARD_SCR)
    c["PROCESSPARAM"]["RES"] = ["f2_1270"]
    res = []
    for ref in (1, 0):
        P = card.build_params(c, "PP[RESTENSOR]<C> -> pi+ pi- @RES{f2_1270:1}")
        P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = 63, 33, 3.0
        e = _engine(P)
        e.eikonal_build(1024, 10000)
        e.set_tuning(fp64_refine=ref)
        vp = _abi.VegasParams()
        vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, 1 << 18, 1.5
        vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, g.MIXED, 7
        e.vegas_init(vp)
        res.append(e.vegas_iteration(mode=0, refine=False, iter_id=1))  # the uniform grid
        e.close()
    print("f2 uniform-grid pass: refined %d, I %.10e (refined) vs %.10e (FP32 only), NaN %d"
          % (res[0].refined, res[0].I_this, res[1].I_this, res[1].nan_count))
    assert res[1].nan_count == 0 and res[1].refined == 0
    assert res[1].I_this == pytest.approx(res[0].I_this, rel=1e-5)

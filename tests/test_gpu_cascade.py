"""Vector-meson pairs with two-body cascades on the GPU through the C ABI: rho rho ->
pi+ pi- pi+ pi- and phi phi -> K+ K- K+ K- in the <F> class (14-dimensional points), the
tensor-pomeron 2xV amplitude and the Regge continuum, against the reference's golden vectors
and the CPU oracle; FP32 kt-loop against FP64; VEGAS integration in 14 dimensions."""
import ctypes
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle_api as orc
from test_gpu_parity import _mixed_ok

pytestmark = pytest.mark.gpu

TOL = 5e-10


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _params(g):
    from graniitti_gb300 import card
    return card.build_params(card.read_card(os.path.join(GOLDEN, "cards", str(g["card"]))),
                             str(g["proc"]))


def _rel(w, wr):
    nz = wr > 0
    assert np.array_equal(w > 0, nz)
    return np.abs(w[nz] - wr[nz]) / wr[nz]


@pytest.mark.parametrize("name", ["rr_tree_weights.npz", "rr_regge_tree_weights.npz",
                                  "ff_tree_weights.npz", "rrc_tree_weights.npz",
                                  "rrc_regge_tree_weights.npz", "rrc14_tree_weights.npz",
                                  "rrf12_tree_weights.npz"])
def test_cascade_tree_vs_reference(gpu, name):
    """<F> and <C> cascades (12 dimensions with @OFFSHELL:0, else 14) against the reference."""
    import graniitti_gb300 as g
    gl = _load(name)
    P = _params(gl)
    e = g.Engine(P, 0)
    assert e.dim == gl["u"].shape[1]
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    wo, flo = orc.weights(P, gl["u"])
    assert np.array_equal(fl, flo) and np.array_equal(fl & 1, gl["kin"])
    kin = gl["kin"] == 1
    assert np.array_equal(((fl >> 1) & 1)[kin], gl["fid"][kin])
    r = _rel(w, gl["w"])
    print("%s: GPU vs reference max rel %.2e, median %.2e (%d weights)" %
          (name, r.max(), np.median(r), r.size))
    assert r.max() < TOL
    assert _rel(w, wo).max() < TOL
    # the central pair (off-shell masses) as the reference has it
    p4, _, _ = e.event_kinematics(gl["u"])
    scale = np.abs(gl["p4"]).max(axis=2, keepdims=True)
    assert (np.abs(p4 - gl["p4"])[kin] / scale[kin]).max() < 1e-12


@pytest.mark.parametrize("name", ["rr_screened_15x12_weights.npz",
                                  "rrc_screened_15x12_weights.npz"])
def test_cascade_screened_vs_reference(gpu, name):
    import graniitti_gb300 as g
    gl = _load(name)
    t = _load("eikonal_nbt1024_nkt10000.npz")
    P = _params(gl)
    e = g.Engine(P, 0)
    e.eikonal_set(t["mbt"], t["msa"])
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    assert np.array_equal(fl & 1, gl["kin"])
    r = _rel(w, gl["w"])
    print("screened rho rho (2xV): GPU FP64 vs reference max rel %.2e" % r.max())
    assert r.max() < 1e-9
    wm, _ = e.event_weights(gl["u"], prec=g.MIXED)
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = g.Engine(Pb, 0).event_weights(gl["u"], prec=g.FP64)
    ok, rel = _mixed_ok(wm, w, wb)
    print("screened rho rho: mixed vs fp64 max rel %.3e" % rel.max())
    assert ok, rel.max()


@pytest.mark.parametrize("proc", [
    "PP[CONTENSOR]<F> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}",
    "PP[CON]<F> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}",
    "PP[CONTENSOR]<C> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-} @OFFSHELL:0"])
def test_cascade_mixed_loop_vs_fp64(gpu, proc):
    """FP32 kt-loop against the FP64 loop on 4096 points (tables built on the device)."""
    import graniitti_gb300 as g
    import philox_np
    from graniitti_gb300 import card
    from conftest import CARD_SCR
    P = card.build_params(card.read_card(CARD_SCR), proc)
    e = g.Engine(P, 0)
    e.eikonal_build()
    u = philox_np.uniforms(85, 4096, e.dim)
    w64, fl = e.event_weights(u, prec=g.FP64)
    wm, flm = e.event_weights(u, prec=g.MIXED)
    assert np.array_equal(fl, flm)
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = g.Engine(Pb, 0).event_weights(u, prec=g.FP64)
    ok, rel = _mixed_ok(wm, w64, wb)
    print("%s: mixed vs fp64 (4096 points, %d screened) max rel %.3e, median %.3e" %
          (proc.split("]")[0], int((w64 > 0).sum()), rel.max(), np.median(rel)))
    assert ok, rel.max()


@pytest.mark.parametrize("name", ["rr_vegas_sigma.json", "rrc_vegas_sigma.json"])
def test_cascade_cross_section_vs_reference_vegas(gpu, name):
    """VEGAS over 14 (<F>) and 12 (<C>, @OFFSHELL:0) dimensions: the tensor-pomeron
    rho rho -> pi+ pi- pi+ pi- cross section against the reference's own VEGAS run."""
    import json
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi, card
    ref = json.load(open(os.path.join(GOLDEN, name)))
    P = card.build_params(card.read_card(os.path.join(GOLDEN, "cards", ref["card"])),
                          ref["process"])
    e = g.Engine(P, 0)
    vp = _abi.VegasParams()
    vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 6, 1 << 20, 1.5
    vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, 0, 5
    r = e.vegas_integrate(vp)
    pull = (r.sigma - ref["sigma_barn"]) / np.hypot(r.sigma_err, ref["sigma_err_barn"])
    print("sigma rho rho (2xV, unscreened): GPU %.5e +- %.1e, reference %.5e +- %.1e, pull %.2f"
          % (r.sigma, r.sigma_err, ref["sigma_barn"], ref["sigma_err_barn"], pull))
    assert abs(pull) < 4


def test_cascade_rejections(gpu):
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi
    gl = _load("rr_tree_weights.npz")
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
    assert status(lambda Q: setattr(Q, "phase_space", _abi.GRN_PS_CONTINUUM)) == _abi.GRN_OK
    assert status(lambda Q: (setattr(Q, "offshell_user", 1), setattr(Q, "offshell", -1.0))) == \
        _abi.GRN_ERR_INVALID
    assert status(lambda Q: setattr(Q, "n_decay", 0)) == _abi.GRN_ERR_UNSUPPORTED
    assert status(lambda Q: setattr(Q, "n_decay", 3)) == _abi.GRN_ERR_UNSUPPORTED
    e = g.Engine(P, 0)
    with pytest.raises(Exception):
        g.Flow(e, hidden=64)  # 14-dimensional flows are built for widths 128 and 256


def test_cascade_events_written(gpu, tmp_path):
    """Unweighted rho rho -> pi+ pi- pi+ pi- events through the driver into HepMC3: six
    vertices, four-momentum conserved, the four pions inside the fiducial cuts."""
    import graniitti_gb300 as g
    from graniitti_gb300.record import read_hepmc3
    from conftest import CARD
    gr = g.Graniitti()
    gr.ReadInput(CARD, "PP[CONTENSOR]<F> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}")
    gr.SetVegasParam(NCALL=1 << 18, ITER=3, PRECISION=0.01)
    gr.Initialize()
    path = str(tmp_path / "rr.hepmc3")
    u, trials, ovf = gr.Generate(200, output=path, fmt="hepmc3")
    assert u.shape == (200, 14)
    ev = read_hepmc3(path)
    assert len(ev) == 200
    for e in ev:
        P = e["particles"]
        assert e["nv"] == 6 and [P[i][1] for i in range(8, 14)] == [113, 113, 211, -211, 211, -211]
        p = {i: P[i][2] for i in P}
        assert np.allclose(p[8], p[10] + p[11], atol=1e-10)
        assert np.allclose(p[9], p[12] + p[13], atol=1e-10)
        assert np.allclose(p[1] + p[4], p[2] + p[5] + p[10] + p[11] + p[12] + p[13], atol=1e-7)
        for i in range(10, 14):
            pt = np.hypot(p[i][0], p[i][1])
            eta = np.arcsinh(p[i][2] / pt)
            assert pt >= 0.1 and abs(eta) <= 0.9

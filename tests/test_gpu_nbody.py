"""Regge continuum of four central particles (PP[CON]<F> -> pi+ pi- pi+ pi-, pi+ pi- K+ K-;
MRegge::ME6 with the weighted N-body phase space of NBodySetup / NBodyPhaseSpace) on the GPU,
against the reference's own weights of the same 14-dimensional points (its generator draws
served from u[6..13]) and its VEGAS cross section."""
import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
# FP64 on both sides; invariants from light-cone components here, from lab 4-vectors in the
# reference (differences at the 1e-11 level of its (q1 - p)^2 with 6.5 TeV beams)
TOL_TREE = 1e-9


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


@pytest.mark.parametrize("name", ["f4_tree_weights.npz", "f4_kk_tree_weights.npz",
                                  "c4_tree_weights.npz"])
def test_four_body_tree_weights_match_reference(gpu, name):
    import graniitti_gb300 as g
    gl = _load(name)
    P = _params(gl)
    e = g.Engine(P, 0)
    assert e.dim == 14
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    assert np.array_equal(fl & 1, gl["kin"])
    kin = gl["kin"] == 1
    assert np.array_equal(((fl >> 1) & 1)[kin], gl["fid"][kin])
    r = _rel(w, gl["w"])
    print("%s: %d of %d points with W > 0, GPU vs reference max rel %.2e median %.2e"
          % (name, (gl["w"] > 0).sum(), len(w), r.max(), np.median(r)))
    assert (gl["w"] > 0).sum() > 50 and r.max() < TOL_TREE
    # a point's weight does not depend on the batch it is evaluated in
    w2, _ = e.event_weights(gl["u"][::-1].copy(), prec=g.FP64)
    assert np.array_equal(w2[::-1], w)
    e.close()


@pytest.mark.parametrize("name", ["f4_screened_weights.npz", "c4_screened_weights.npz"])
def test_four_body_screened_weights_match_reference(gpu, name):
    import graniitti_gb300 as g
    gl = _load(name)
    t = _load("eikonal_nbt1024_nkt10000.npz")
    P = _params(gl)
    assert P.screening
    e = g.Engine(P, 0)
    e.eikonal_set(t["mbt"], t["msa"])
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    assert np.array_equal(fl & 1, gl["kin"])
    r = _rel(w, gl["w"])
    print("%s: GPU FP64 vs reference max rel %.2e" % (name, r.max()))
    assert r.max() < 1e-9
    # MIXED: the FP32 4-body loop, events whose error estimate exceeds 1e-5 redone in FP64
    wm, _ = e.event_weights(gl["u"], prec=g.MIXED)
    rm = _rel(wm, gl["w"])
    e.set_tuning(fp64_refine=0)
    w32, _ = e.event_weights(gl["u"], prec=g.MIXED)
    r32 = _rel(w32, gl["w"])
    print("%s: GPU MIXED vs reference max rel %.2e (FP32 loop alone %.2e)"
          % (name, rm.max(), r32.max()))
    assert rm.max() < 1e-5
    # the FP32 loop ran: its weights are not the FP64 ones
    assert not np.array_equal(w32, w)
    e.close()


@pytest.mark.parametrize("card_name", ["f4_screened", "c4_screened"])
def test_four_body_fp32_loop_vs_fp64(gpu, card_name):
    """The FP32 4-body loop with FP64 refinement against the FP64 loop over 2^14 seeded
    points: relative weight difference below 1e-5 on every point (the refinement bound)."""
    import graniitti_gb300 as g
    import philox_np
    gl = _load(card_name + "_weights.npz")
    t = _load("eikonal_nbt1024_nkt10000.npz")
    P = _params(gl)
    e = g.Engine(P, 0)
    e.eikonal_set(t["mbt"], t["msa"])
    u = philox_np.uniforms(91, 1 << 14, 14)
    w64, fl = e.event_weights(u, prec=g.FP64)
    wm, flm = e.event_weights(u, prec=g.MIXED)
    assert np.array_equal(fl, flm)
    nz = w64 > 0
    assert nz.sum() > 500 and np.array_equal(wm > 0, nz)
    r = np.abs(wm[nz] - w64[nz]) / w64[nz]
    print("%s: MIXED vs FP64 over %d points with W > 0: max rel %.2e, median %.2e"
          % (card_name, nz.sum(), r.max(), np.median(r)))
    assert r.max() < 1e-5
    e.close()


def test_four_body_vegas_cross_section(gpu):
    """sigma(pp -> p pi+ pi- pi+ pi- p) with the fiducial cuts of the card: GPU VEGAS over the
    14-dimensional hypercube vs the mean of the reference's own EventWeight over 4e6 uniform
    points (its generator draws). The integrand is heavy-tailed; the reference's VEGAS over
    its 6 dimensions reports 1.67e-10 b +- 0.1%, a factor 8 below that mean, and is recorded
    in the fixture but not used."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi, card
    ref = json.load(open(os.path.join(GOLDEN, "f4_sigma.json")))
    P = card.build_params(card.read_card(os.path.join(GOLDEN, "cards", ref["card"])),
                          ref["process"])
    e = g.Engine(P, 0)
    vp = _abi.VegasParams()
    vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, 1 << 22, 1.5
    vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 5e-4, 3, g.FP64, 11
    e.vegas_init(vp)
    for it in range(8):
        e.vegas_iteration(mode=0, refine=True, iter_id=it)
    e.vegas_clear()
    r = None
    for it in range(6):
        r = e.vegas_iteration(mode=1, refine=True, iter_id=20 + it)
    ref_s, ref_e = ref["flat_sigma_barn"], ref["flat_sigma_err_barn"]
    pull = (r.sigma - ref_s) / np.hypot(r.sigma_err, ref_e)
    print("4 pi sigma: GPU VEGAS %.5e +- %.1e b, reference EventWeight flat mean %.5e +- %.1e b "
          "(%d points), pull %.2f" % (r.sigma, r.sigma_err, ref_s, ref_e, ref["flat_points"],
                                      pull))
    assert r.sigma_err / r.sigma < 1e-2 and abs(pull) < 4
    e.close()


def test_four_body_histograms(gpu):
    """On-the-fly histograms of a 4-body pass: the system observables and the angles of the
    first central particle, against the oracle's observables of the same points."""
    import graniitti_gb300 as g
    from test_gpu_histograms import _compare, _vegas
    from graniitti_gb300 import card
    from conftest import CARD
    P = card.build_params(card.read_card(CARD), "PP[CON]<F> -> pi+ pi- pi+ pi-")
    e = g.Engine(P, 0)
    _vegas(e, g, ncall=1 << 15)
    f = e.pass_weights(1 << 15)
    specs = [("M", 30, 0.5, 5.0), ("Y", 18, -0.9, 0.9), ("PT", 20, 0.0, 2.0),
             ("RAP3", 20, -1.0, 1.0), ("COSTH_CS", 10, -1.0, 1.0, "PHI_CS", 10, -np.pi, np.pi),
             ("COSTH_LA", 20, -1.0, 1.0)]
    e.hist_define(specs)
    e.hist_clear()
    e.hist_fill()
    _compare(e, P, specs, f)
    e.close()


def test_four_body_record_kinematics_and_events(gpu, tmp_path):
    """Forward legs and the four central particles against the reference's pfinal of the same
    points, and the HepMC3 record (CommonRecord: system -> four stable particles)."""
    import graniitti_gb300 as g
    from graniitti_gb300.record import EventWriter
    gl = _load("f4_tree_weights.npz")
    e = g.Engine(_params(gl), 0)
    p4, ts, fl = e.event_kinematics(gl["u"])
    kin = gl["kin"] == 1
    assert np.array_equal(fl & 1, gl["kin"])
    scale = np.abs(gl["p4"]).max(axis=2, keepdims=True)
    assert (np.abs(p4 - gl["p4"])[kin] / scale[kin]).max() < 1e-11
    pd = e.event_daughters(gl["u"])
    sc = np.abs(gl["leaves"]).max(axis=2, keepdims=True)
    assert (np.abs(pd - gl["leaves"])[kin] / sc[kin]).max() < 1e-11
    assert np.allclose(ts[kin, 0], gl["t1"][kin], rtol=1e-6)
    path = str(tmp_path / "f4.hepmc3")
    idx = np.nonzero(gl["w"] > 0)[0][:20]
    with EventWriter(path, "hepmc3") as w:
        n = w.write_points(e, gl["u"][idx], [2212, 211, -211, 211, -211], 1.0, 0.1)
    assert n == len(idx)
    parts = [l.split() for l in open(path) if l.startswith("P ")]
    assert len(parts) == 11 * len(idx)
    last = np.array([[float(v) for v in p[4:8]] for p in parts]).reshape(len(idx), 11, 4)[:, 7:]
    assert np.allclose(last, pd[idx], rtol=1e-12, atol=1e-12)
    assert [int(p[3]) for p in parts[7:11]] == [211, -211, 211, -211]
    e.close()


@pytest.mark.parametrize("name", ["veto_c_weights.npz", "veto_rr_weights.npz",
                                  "veto_f4_weights.npz"])
def test_veto_cuts_match_reference(gpu, name):
    """Veto cuts (two domains on the final-state leaves) for a 2-body continuum, a cascade
    and a 4-body state: veto flags and weights as the reference's."""
    import graniitti_gb300 as g
    gl = _load(name)
    e = g.Engine(_params(gl), 0)
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    kin = gl["kin"] == 1
    assert np.array_equal(fl & 1, gl["kin"])
    assert np.array_equal(((fl >> 2) & 1)[kin], gl["veto"][kin])
    r = _rel(w, gl["w"])
    print("%s: %d vetoed, GPU vs reference max rel %.2e" % (name, (gl["veto"][kin] == 0).sum(),
                                                           r.max()))
    assert r.max() < 1e-9
    e.close()

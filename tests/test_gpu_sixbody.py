"""Regge continuum of six central particles (PP[CON]<F|C> -> pi+ pi- pi+ pi- pi+ pi-,
MRegge::ME8 over the 720 ladder orderings) on the GPU, against the reference's own weights of
the same 20-dimensional points (its generator draws served from the point through the RNG
replay) and the long-double oracle."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
# FP64 on both sides: light-cone invariants here, lab 4-vectors in the reference
TOL_REF = 1e-9
# against the oracle restatement evaluated in long double
TOL_LD = 1e-10


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


def _ld(P, u, msa=None):
    from oracle import oracle_api as orc
    w, _ = orc.weights(P, u, msa=msa, nthreads=16, long_double=True)
    return w


@pytest.mark.parametrize("name", ["f6_tree_weights.npz", "c6_tree_weights.npz"])
def test_six_body_tree_weights_match_reference(gpu, name):
    import graniitti_gb300 as g
    gl = _load(name)
    P = _params(gl)
    e = g.Engine(P, 0)
    assert e.dim == 20
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    assert np.array_equal(fl & 1, gl["kin"])
    kin = gl["kin"] == 1
    assert np.array_equal(((fl >> 1) & 1)[kin], gl["fid"][kin])
    r = _rel(w, gl["w"])
    rl = _rel(w, _ld(P, gl["u"]))
    print("%s: %d of %d points with W > 0, GPU vs reference max rel %.2e, vs long double %.2e"
          % (name, (gl["w"] > 0).sum(), len(w), r.max(), rl.max()))
    assert (gl["w"] > 0).sum() > 40 and r.max() < TOL_REF and rl.max() < TOL_LD
    e.close()


@pytest.mark.parametrize("name", ["f6_screened_weights.npz", "c6_screened_weights.npz"])
def test_six_body_screened_weights_match_reference(gpu, name):
    """FP64 loop against the reference and the long-double oracle; MIXED (the FP64 loop with
    FP32 loop nodes: no FP32 6-body loop exists) against the reference."""
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
    rl = _rel(w, _ld(P, gl["u"], t["msa"]))
    wm, _ = e.event_weights(gl["u"], prec=g.MIXED)
    rm = _rel(wm, gl["w"])
    print("%s: %d screened, GPU FP64 vs reference max rel %.2e, vs long double %.2e; "
          "MIXED vs reference %.2e" % (name, (gl["w"] > 0).sum(), r.max(), rl.max(), rm.max()))
    assert (gl["w"] > 0).sum() >= 20
    assert r.max() < TOL_REF and rl.max() < TOL_LD and rm.max() < 1e-5
    e.close()


def test_six_body_daughters_and_records(gpu, tmp_path):
    """The six central particles against the reference's pfinal[3..8] of the same points, and
    the HepMC3 record (system -> six stable particles)."""
    import graniitti_gb300 as g
    from graniitti_gb300.record import EventWriter
    gl = _load("c6_tree_weights.npz")
    e = g.Engine(_params(gl), 0)
    p4, ts, fl = e.event_kinematics(gl["u"])
    kin = gl["kin"] == 1
    scale = np.abs(gl["p4"]).max(axis=2, keepdims=True)
    assert (np.abs(p4 - gl["p4"])[kin] / scale[kin]).max() < 1e-11
    pd = e.event_daughters(gl["u"])
    assert pd.shape == (len(gl["u"]), 6, 4)
    sc = np.abs(gl["leaves"]).max(axis=2, keepdims=True)
    assert (np.abs(pd - gl["leaves"])[kin] / sc[kin]).max() < 1e-11
    path = str(tmp_path / "c6.hepmc3")
    idx = np.nonzero(gl["w"] > 0)[0][:20]
    with EventWriter(path, "hepmc3") as w:
        n = w.write_points(e, gl["u"][idx], [2212, 211, -211, 211, -211, 211, -211], 1.0, 0.1)
    assert n == len(idx)
    parts = [l.split() for l in open(path) if l.startswith("P ")]
    assert len(parts) == 13 * len(idx)
    last = np.array([[float(v) for v in p[4:8]] for p in parts]).reshape(len(idx), 13, 4)[:, 7:]
    assert np.allclose(last, pd[idx], rtol=1e-12, atol=1e-12)
    assert [int(p[3]) for p in parts[7:13]] == [211, -211, 211, -211, 211, -211]
    e.close()


def test_six_body_vegas_passes(gpu):
    """VEGAS over the 20-dimensional hypercube (continuum class, tree level, FP64): the grid
    adapts, and the same seed gives the same grid and integral (the fixed-order histogram
    holds the bins of 20 dimensions). The integrand is extremely heavy-tailed over the card's
    rapidity range of +-9 per particle, so no flat-sampling cross check is made."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi
    gl = _load("c6_tree_weights.npz")
    res = []
    for rep in range(2):
        e = g.Engine(_params(gl), 0)
        vp = _abi.VegasParams()
        vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, 1 << 18, 1.5
        vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, g.FP64, 5
        e.vegas_init(vp)
        for it in range(3):
            e.vegas_iteration(mode=0, refine=True, iter_id=1 + it)
        e.vegas_clear()
        r = [e.vegas_iteration(mode=1, refine=True, iter_id=10 + it) for it in range(2)][-1]
        res.append((r.sigma, r.sigma_err, e.vegas_grid()))
        e.close()
    s, se, grid = res[0]
    print("6 pi <C> tree: VEGAS %.5e +- %.1e b" % (s, se))
    assert res[0][0] == res[1][0] and np.array_equal(res[0][2], res[1][2])
    assert np.isfinite(s) and s > 0 and np.isfinite(se)
    uniform = np.arange(1, 129)[:, None] / 128.0
    assert np.abs(grid - uniform).max() > 1e-3  # the grid adapted

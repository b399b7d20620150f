"""On-the-fly histograms (grn_hist_*): the GPU fills the reference's level-1/2 observables
(MUserHistograms::FillHistograms, src/MUserHistograms.cc:60-125) from the points and weights of
the last pass; the oracle computes the same observables from the same hypercube points on
the CPU (orc_observables) and numpy bins them with the same weights."""
import numpy as np
import pytest

from oracle import oracle_api as orc

pytestmark = pytest.mark.gpu

RHO = "PP[CONTENSOR]<F> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}"
SPECS = [
    ("M", 40, 0.3, 3.0),
    ("Y", 24, -1.2, 1.2),
    ("PT", 30, 0.0, 1.5),
    ("DPHI_PP", 18, 0.0, np.pi),
    ("PT1", 25, 0.0, 1.0),
    ("RAP3", 20, -1.0, 1.0),
    ("COSTH_CS", 10, -1.0, 1.0, "PHI_CS", 12, -np.pi, np.pi),
    ("COSTH_HX", 20, -1.0, 1.0),
    ("PHI_HX", 20, -np.pi, np.pi),
    ("COSTH_AH", 20, -1.0, 1.0),
    ("COSTH_PG", 20, -1.0, 1.0, "PHI_PG", 8, -np.pi, np.pi),
    ("COSTH_CM", 20, -1.0, 1.0),
    ("PHI_CM", 20, -np.pi, np.pi),
    ("COSTH_LA", 20, -1.0, 1.0),
    ("PHI_LA", 16, -np.pi, np.pi),
]
EDGE = 1e-9  # an observable this close (relative to the bin width) to an edge may fall either side


def _bin(v, n, lo, hi):
    """hist_bin of the fill kernel: -3 NaN, -1 below, -2 at or above hi, else the bin; and
    whether v is within EDGE bin widths of an edge."""
    k = np.full(v.shape, -3, dtype=np.int64)
    ok = ~np.isnan(v)
    k[ok & (v < lo)] = -1
    k[ok & (v >= hi)] = -2
    inside = ok & (v >= lo) & (v < hi)
    t = (v[inside] - lo) / (hi - lo) * n
    k[inside] = np.minimum(t.astype(np.int64), n - 1)
    near = np.zeros(v.shape, dtype=bool)
    tt = (v[ok] - lo) / (hi - lo) * n
    near[ok] = np.abs(tt - np.round(tt)) < EDGE * max(1.0, n)
    return k, near


def _reference_hist(spec, obs, f):
    names = orc_names()
    k, near = _bin(obs[:, names.index(spec[0])], spec[1], spec[2], spec[3])
    nb = spec[1]
    if len(spec) > 4:
        k2, near2 = _bin(obs[:, names.index(spec[4])], spec[5], spec[6], spec[7])
        k = np.where(k < 0, k, np.where(k2 < 0, k2, k * spec[5] + k2))
        near |= near2
        nb *= spec[5]
    w = np.zeros(nb)
    w2 = np.zeros(nb)
    c = np.zeros(nb, dtype=np.int64)
    inb = k >= 0
    np.add.at(w, k[inb], f[inb])
    np.add.at(w2, k[inb], f[inb] ** 2)
    np.add.at(c, k[inb], 1)
    out = np.array([(k == -1).sum(), (k == -2).sum(), (k == -3).sum()])
    return w, w2, c, out, near


def orc_names():
    from graniitti_gb300 import _abi
    return _abi.OBS


def _compare(e, params, specs, f, fill_count=1, scale_f=1.0):
    idx = np.nonzero(f > 0)[0]
    u = e.vegas_points(idx)
    obs, ok = orc.observables(params, u)
    assert ok.all(), "a point with f > 0 fails the oracle's kinematics"
    fw = f[idx] * scale_f
    for h, spec in enumerate(specs):
        w, w2, c, out = e.hist_get(h)
        rw, rw2, rc, rout, near = _reference_hist(spec, obs, fw)
        amb = int(near.sum())
        dc = np.abs(c.ravel() - fill_count * rc).sum()
        # + 1 point: the anti-helicity axis (nearly opposite beams summed) is ill-conditioned
        assert dc <= 2 * fill_count * (amb + 1), (spec, dc, amb)
        assert np.abs(out - fill_count * rout).sum() <= 2 * fill_count * (amb + 1), (spec, out)
        slack = fw[near].sum() + fw.max()
        tol = 1e-9 * fill_count * fw.sum() + 2 * fill_count * slack
        assert np.abs(w.ravel() - fill_count * rw).max() <= tol, spec
        tol2 = 1e-9 * fill_count * (fw ** 2).sum() + 2 * fill_count * ((fw[near] ** 2).sum()
                                                                       + fw.max() ** 2)
        assert np.abs(w2.ravel() - fill_count * rw2).max() <= tol2, spec
        assert c.sum() + out.sum() == fill_count * len(idx)
    return obs


def _vegas(e, g, ncall=1 << 16, seed=5, iters=3):
    from graniitti_gb300 import _abi
    vp = _abi.VegasParams()
    vp.bins, vp.iter, vp.ncall, vp.lambda_ = 64, 3, ncall, 1.5
    vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, g.FP64, seed
    e.vegas_init(vp)
    for it in range(iters):
        e.vegas_iteration(mode=0, refine=True, iter_id=it)
    return e.vegas_iteration(mode=1, refine=False, iter_id=20)


def test_histograms_of_a_vegas_pass_match_oracle_observables(gpu, params):
    import graniitti_gb300 as g
    e = g.Engine(params, 0)
    _vegas(e, g)
    n = 1 << 16
    f = e.pass_weights(n)
    assert (f > 0).sum() > n // 4
    e.hist_define(SPECS)
    e.hist_clear()
    e.hist_fill()
    obs = _compare(e, params, SPECS, f)
    cols = [orc_names().index(c) for c in ("COSTH_CS", "COSTH_HX", "COSTH_AH", "COSTH_PG",
                                          "COSTH_CM", "COSTH_LA")]
    assert np.all(np.abs(obs[:, cols]) <= 1 + 1e-12)
    # a second fill adds the same pass again
    e.hist_fill()
    _compare(e, params, SPECS, f, fill_count=2)
    e.hist_clear()
    w, w2, c, out = e.hist_get(0)
    assert not w.any() and not c.any() and not out.any()
    e.close()


def test_histograms_of_a_cascade_pass(gpu):
    """rho rho -> pi+ pi- pi+ pi- (14-dimensional hypercube): M0 (the sampled rho mass) and
    the rho rapidities."""
    import graniitti_gb300 as g
    from graniitti_gb300 import card
    from conftest import CARD
    P = card.build_params(card.read_card(CARD), RHO)
    e = g.Engine(P, 0)
    _vegas(e, g, ncall=1 << 15)
    f = e.pass_weights(1 << 15)
    specs = [("M", 30, 1.0, 3.0), ("M0", 40, 0.3, 1.3), ("RAP3", 20, -1.0, 1.0),
             ("RAP4", 20, -1.0, 1.0), ("COSTH_HX", 10, -1.0, 1.0, "PHI_HX", 10, -np.pi, np.pi)]
    e.hist_define(specs)
    e.hist_clear()
    e.hist_fill()
    _compare(e, P, specs, f)
    e.close()


def test_histograms_of_a_flow_pass(gpu, params):
    """Flow passes fill from the flow's points (the weights include 1 / q)."""
    import graniitti_gb300 as g
    e = g.Engine(params, 0)
    _vegas(e, g, ncall=1 << 15)
    fl = g.Flow(e, layers=6, seed=3)
    fl.iteration(mode=1, iter_id=40)
    f = e.pass_weights(1 << 15)
    e.hist_define(SPECS[:4])
    e.hist_clear()
    e.hist_fill()
    _compare(e, params, SPECS[:4], f)
    fl.close()
    e.close()

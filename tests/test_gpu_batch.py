"""Several processes in one pass (grn_batch): the fused, graph-replayed pass gives each
process exactly the pass it gets alone, and a batched integration the same cross sections."""
import ctypes

import numpy as np
import pytest

from conftest import CARD_SCR

pytestmark = pytest.mark.gpu


def _engines(n_call):
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi, card
    c = card.read_card(CARD_SCR)
    procs = ["PP[CON]<C> -> pi+ pi-", "PP[CON]<C> -> K+ K-", "PP[CONTENSOR]<C> -> pi+ pi-"]
    out = []
    for k, proc in enumerate(procs):
        P = card.build_params(c, proc)
        P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = 15, 12, 1.75
        e = g.Engine(P, 0)
        e.eikonal_build(512, 2000)
        e.set_tuning(loop_pair=1)
        vp = _abi.VegasParams()
        vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, n_call[k], 1.5
        vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, g.MIXED, 11 + k
        e.vegas_init(vp)
        out.append(e)
    return out


def test_batched_pass_equals_separate_passes(gpu):
    import graniitti_gb300 as g
    calls = [1 << 16, 3 << 14, 1 << 15]
    es = _engines(calls)
    grids = [e.vegas_grid() for e in es]
    sep = [e.vegas_iteration(mode=1, refine=False, iter_id=7) for e in es]
    for e, x in zip(es, grids):
        e.vegas_clear()
        e.vegas_set_grid(x)
    b = g.Batch(es)
    res, ms = b.iteration(mode=1, refine=False, iter_id=7)
    for r0, r1 in zip(sep, res):
        # the engines' counters accumulate over both passes
        assert r1.evaluations == 2 * r0.evaluations and r1.kinematics_ok == 2 * r0.kinematics_ok
        assert r1.amplitude_ok == 2 * r0.amplitude_ok and r1.nan_count == 2 * r0.nan_count
        assert r1.I_this == pytest.approx(r0.I_this, rel=1e-14)
        assert r1.maxf == pytest.approx(r0.maxf, rel=1e-14)
    print("batched pass of 3 processes: %.2f ms; I = %s" % (ms, [r.I_this for r in res]))
    # an engine in a batch cannot be destroyed
    with pytest.raises(Exception):
        from graniitti_gb300 import _abi
        _abi.check(es[0].lib.grn_destroy(es[0].h))
    b.close()
    for e in es:
        e.close()


def test_batched_integration_matches_separate(gpu):
    import graniitti_gb300 as g
    calls = [1 << 16, 1 << 16, 1 << 16]
    es = _engines(calls)
    b = g.Batch(es)
    for it in range(4):
        b.iteration(mode=0, refine=True, iter_id=100 + it)
    for e in es:
        e.vegas_clear()
    for it in range(6):
        res, ms = b.iteration(mode=1, refine=True, iter_id=200 + it)
    b.close()
    sep = []
    for e in _engines(calls):
        for it in range(4):
            e.vegas_iteration(mode=0, refine=True, iter_id=300 + it)
        e.vegas_clear()
        for it in range(6):
            r = e.vegas_iteration(mode=1, refine=True, iter_id=400 + it)
        sep.append(r)
    for rb, rs in zip(res, sep):
        pull = (rb.sigma - rs.sigma) / np.hypot(rb.sigma_err, rs.sigma_err)
        print("batched %.5e +- %.1e vs separate %.5e +- %.1e: pull %.2f"
              % (rb.sigma, rb.sigma_err, rs.sigma, rs.sigma_err, pull))
        assert abs(pull) < 4
    for e in es:
        e.close()


def test_batched_mixed_multiplicity_equals_separate(gpu):
    """The mixed workload of uneven multiplicity: tensor-pomeron f2(1270) -> pi+ pi- (2-body),
    the Regge pi+ pi- continuum (2-body, record mode) and tensor-pomeron rho rho ->
    pi+ pi- pi+ pi- (4-body, 14 dimensions), 50/30/20, screened, in one batched pass."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi, card
    c = card.read_card(CARD_SCR)
    c["GENCUTS"]["<F>"]["M"] = [0.5, 3.0]
    c["PROCESSPARAM"]["RES"] = ["f2_1270"]
    procs = ["PP[RESTENSOR]<F> -> pi+ pi-", "PP[CON]<C> -> pi+ pi-",
             "PP[CONTENSOR]<F> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}"]
    total = 1 << 17
    calls = [total // 2, 3 * total // 10, total - total // 2 - 3 * total // 10]
    es = []
    for k, proc in enumerate(procs):
        P = card.build_params(c, proc)
        e = g.Engine(P, 0)
        e.eikonal_build(512, 2000)
        e.set_tuning(loop_pair=1)  # the batched record-mode loop pairs events
        vp = _abi.VegasParams()
        vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, calls[k], 1.5
        vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, g.MIXED, 31 + k
        e.vegas_init(vp)
        es.append(e)
    assert [e.dim for e in es] == [8, 8, 14]
    grids = [e.vegas_grid() for e in es]
    sep = [e.vegas_iteration(mode=1, refine=False, iter_id=9) for e in es]
    for e, x in zip(es, grids):
        e.vegas_clear()
        e.vegas_set_grid(x)
    b = g.Batch(es)
    res, ms = b.iteration(mode=1, refine=False, iter_id=9)
    for r0, r1 in zip(sep, res):
        assert r1.evaluations == 2 * r0.evaluations and r1.fidcuts_ok == 2 * r0.fidcuts_ok
        assert r1.I_this == pytest.approx(r0.I_this, rel=1e-14)
        assert r1.maxf == pytest.approx(r0.maxf, rel=1e-14)
    print("batched 2-body + 4-body pass: %.2f ms; I = %s" % (ms, [r.I_this for r in res]))
    b.close()
    # a refined pass: the batched graph builds each member's f^2 histogram in the same fixed
    # order as the engine alone (and every member's points get the same weights, the record-
    # mode member on the same paired loop kernel), so the refined grids are equal bit for bit
    for e, x in zip(es, grids):
        e.vegas_set_grid(x)
    sep = [e.vegas_iteration(mode=1, refine=True, iter_id=10) for e in es]
    new_sep = [e.vegas_grid() for e in es]
    for e, x in zip(es, grids):
        e.vegas_set_grid(x)
    b = g.Batch(es)
    res, _ = b.iteration(mode=1, refine=True, iter_id=10)
    b.close()
    for e, x, r0, r1 in zip(es, new_sep, sep, res):
        assert np.array_equal(e.vegas_grid(), x)
        assert r1.I_this == r0.I_this and r1.maxf == r0.maxf
    for e in es:
        e.close()


def test_batched_flow_member_equals_flow_iteration(gpu):
    """A member with a flow proposal (rho rho -> 4 pi, 14 dimensions, 8 layers of width 256)
    gets in the batched pass exactly the pass grn_flow_iteration gives it alone; the flow
    cannot be destroyed while the batch holds it."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi, card
    from oracle import flow_ref as F
    c = card.read_card(CARD_SCR)
    procs = ["PP[CON]<C> -> pi+ pi-",
             "PP[CONTENSOR]<F> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}"]
    es = []
    for k, proc in enumerate(procs):
        e = g.Engine(card.build_params(c, proc), 0)
        e.eikonal_build(512, 2000)
        e.set_tuning(loop_pair=1)  # the batched record-mode loop pairs events
        vp = _abi.VegasParams()
        vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, 1 << 15, 1.5
        vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, g.MIXED, 41 + k
        e.vegas_init(vp)
        es.append(e)
    f = g.Flow(es[1], layers=8, hidden=256, seed=3, mix_uniform=0.1)
    th = F.init_params(dim=14, layers=8, hidden=256, seed=3)
    rng = np.random.default_rng(4)
    for p in F.unpack(th, 14, 8, 256, 16):
        p["W3"] += rng.normal(0, 0.02, p["W3"].shape)
        p["b3"] += rng.normal(0, 0.2, p["b3"].shape)
    f.set_params(th.astype(np.float32))
    grids = [e.vegas_grid() for e in es]
    sep = [es[0].vegas_iteration(mode=1, refine=False, iter_id=5), f.iteration(mode=1, iter_id=5)]
    for e, x in zip(es, grids):
        e.vegas_clear()
        e.vegas_set_grid(x)
    b = g.Batch(es)
    b.set_flow(1, f)
    with pytest.raises(Exception):
        _abi.check(f.lib.grn_flow_destroy(f.h))
    res, ms = b.iteration(mode=1, refine=False, iter_id=5)
    for r0, r1 in zip(sep, res):
        assert r1.I_this == pytest.approx(r0.I_this, rel=1e-14)
        assert r1.maxf == pytest.approx(r0.maxf, rel=1e-14)
    print("batched pass with a flow member: %.2f ms; I = %s" % (ms, [r.I_this for r in res]))
    b.close()
    f.close()
    for e in es:
        e.close()

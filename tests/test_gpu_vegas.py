"""VEGAS on the GPU: one pass against a CPU replay with the oracle, the
integrated cross section against the reference's, and unweighting."""
import json
import os

import numpy as np
import pytest

import philox_np
from conftest import GOLDEN
from oracle import oracle_api as orc

pytestmark = pytest.mark.gpu


def _vp(ncall, prec=0, seed=3, bins=128, iters=5, precision=1e-3):
    from graniitti_gb300 import _abi
    vp = _abi.VegasParams()
    vp.bins, vp.iter, vp.ncall, vp.lambda_ = bins, iters, ncall, 1.5
    vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, precision, 3, prec, seed
    return vp


def test_one_pass_matches_cpu_replay(gpu, params):
    import graniitti_gb300 as g
    n = 1 << 15
    e = g.Engine(params, 0)
    vp = _vp(n)
    e.vegas_init(vp)
    x0 = e.vegas_grid()
    r = e.vegas_iteration(mode=1, refine=True, iter_id=5)
    x1 = e.vegas_grid()
    # CPU replay: same Philox points, oracle map + weights, histogram, refine
    u = philox_np.uniforms(3, n, 8, stream=5)
    xs, vw, bins = orc.vegas_map(x0, u)
    w, fl = orc.weights(params, xs, nthreads=16)
    f = w * vw
    f2 = np.zeros((128, 8))
    for j in range(8):
        np.add.at(f2[:, j], bins[:, j] - 1, f * f)
    assert abs(r.I_this / f.mean() - 1) < 1e-9
    assert abs(r.maxf / f.max() - 1) < 1e-9
    assert r.evaluations == n and r.kinematics_ok == (fl & 1).sum()
    assert r.fidcuts_ok == ((fl >> 1) & 1).sum()
    x1_cpu = orc.vegas_refine(x0, f2)
    assert np.max(np.abs(x1 - x1_cpu)) < 1e-9
    # regenerated points of the pass are the mapped points
    idx = np.array([0, 17, n - 1])
    assert np.allclose(e.vegas_points(idx), xs[idx], rtol=0, atol=1e-15)


def test_cross_section_vs_reference(gpu, params):
    """FP64 GPU VEGAS cross section vs the reference's own VEGAS run (ranlux48
    points, 8 threads): agreement within the combined statistical error."""
    import graniitti_gb300 as g
    ref = json.load(open(os.path.join(GOLDEN, "c1_vegas_sigma.json")))
    e = g.Engine(params, 0)
    r = e.vegas_integrate(_vp(1 << 20, precision=5e-4))
    comb = np.hypot(r.sigma_err, ref["sigma_err_barn"])
    pull = (r.sigma - ref["sigma_barn"]) / comb
    print("sigma gpu %.6e +- %.2e, ref %.6e +- %.2e, pull %.2f" %
          (r.sigma, r.sigma_err, ref["sigma_barn"], ref["sigma_err_barn"], pull))
    assert abs(pull) < 4.0
    assert r.sigma_err / r.sigma < 5e-4


def test_unweighting_matches_recomputation(gpu, params):
    import graniitti_gb300 as g
    n = 1 << 16
    e = g.Engine(params, 0)
    e.vegas_init(_vp(n))
    r = e.vegas_iteration(mode=1, refine=False, iter_id=9)
    x0 = e.vegas_grid()
    u = philox_np.uniforms(3, n, 8, stream=9)
    xs, vw, _ = orc.vegas_map(x0, u)
    w, _ = orc.weights(params, xs, nthreads=16)
    f = w * vw
    fmax = 0.5 * r.maxf  # force some overflow
    na, no, idx = e.unweight(fmax, seed=21, cap=n)
    # the acceptance uniforms: Philox key = seed, block 0 of stream 0x80000000 | iter
    U = philox_np.uniforms(21, n, 2, stream=0x80000000 | 9)[:, 0]
    ovf = f > fmax
    hit = (~ovf) & (U < f / fmax)
    assert na == hit.sum() and no == ovf.sum()
    assert np.array_equal(idx, np.nonzero(hit)[0])


def test_mixed_precision_vegas_screened(gpu, params_screened):
    """Screened VEGAS pass in mixed precision vs the FP64 pass on the same points."""
    import graniitti_gb300 as g
    P = params_screened
    P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = 63, 33, 3.0
    n = 1 << 14
    res = {}
    for prec in (g.FP64, g.MIXED):
        e = g.Engine(P, 0)
        e.eikonal_build(1024, 10000)
        e.vegas_init(_vp(n, prec=prec))
        res[prec] = e.vegas_iteration(mode=1, refine=False, iter_id=4)
    assert abs(res[g.MIXED].I_this / res[g.FP64].I_this - 1) < 2e-6


@pytest.mark.parametrize("proc", ["PP[CON]<C> -> pi+ pi-", "PP[CONTENSOR]<C> -> pi+ pi-"])
def test_refined_grid_bit_reproducible(gpu, proc):
    """Two engines with the same seed give bit-identical grids, integrals and maxima after
    refined passes: the screened work list is filled in a different order each time (record
    mode for the Regge continuum, the FP32 loop with its FP64 refinement list for the tensor
    pomeron), but the f^2 histogram of the refinement is summed in a fixed order."""
    import graniitti_gb300 as g
    from graniitti_gb300 import card
    from conftest import CARD_SCR
    runs = []
    for rep in range(2):
        P = card.build_params(card.read_card(CARD_SCR), proc)
        P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = 15, 12, 1.75
        e = g.Engine(P, 0)
        e.eikonal_build(512, 2000)
        e.vegas_init(_vp(1 << 16, prec=g.MIXED, seed=77))
        res = [e.vegas_iteration(mode=1, refine=True, iter_id=1 + it) for it in range(3)]
        runs.append((e.vegas_grid(), res))
        e.close()
    (x0, r0), (x1, r1) = runs
    assert np.array_equal(x0, x1)
    for a, b in zip(r0, r1):
        assert a.I_this == b.I_this and a.I2_this == b.I2_this and a.maxf == b.maxf
    assert r0[-1].sigma == r1[-1].sigma

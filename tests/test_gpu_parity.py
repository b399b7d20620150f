"""GPU parity through the C ABI: the CUDA path against the reference's golden
vectors and against the CPU oracle on the same seeded inputs."""
import os

import numpy as np
import pytest

import philox_np
from conftest import GOLDEN
from oracle import oracle_api as orc

pytestmark = pytest.mark.gpu

# FP64 path: the GPU's light-cone formulation vs the reference's 4-vector one.
TOL_FP64_REF = 5e-10
TOL_FP64_ORC = 5e-10
# FP32 kt-loop with compensated sums vs FP64: 1e-5 relative. Near exact screening
# dips (|A0 + A_loop|^2 <= 1% of |A0|^2) the absolute error of the loop sum is
# amplified by the cancellation, so the bound carries a floor of 1e-7 of the
# unscreened (Born) weight of the same point.
TOL_MIXED = 1e-5
FLOOR_BORN = 1e-7


def _mixed_ok(wm, w64, wborn):
    err = np.abs(wm - w64)
    bound = TOL_MIXED * np.abs(w64) + FLOOR_BORN * np.abs(wborn)
    nz = w64 > 0
    rel = err[nz] / w64[nz]
    return bool(np.all(err <= bound)), rel


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _engine(P):
    import graniitti_gb300 as g
    return g.Engine(P, 0)


def _rel(w, wr):
    nz = wr > 0
    assert np.array_equal(w > 0, nz)
    return np.abs(w[nz] - wr[nz]) / wr[nz]


def test_uniforms_bit_exact(gpu, params):
    e = _engine(params)
    a = e.uniforms(seed=0xDEADBEEF12345, n=100000, first=(1 << 40) + 3, stream=77)
    b = philox_np.uniforms(0xDEADBEEF12345, 100000, 8, first=(1 << 40) + 3, stream=77)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("name,ff", [("c1_tune0_weights.npz", 2), ("c1_expff_weights.npz", 0),
                                     ("c1_orearff_weights.npz", 1), ("c1_edge_weights.npz", 2)])
def test_tree_weights_vs_reference(gpu, params, name, ff):
    import graniitti_gb300 as g
    gl = _load(name)
    params.regge.offshellFF = ff
    try:
        e = _engine(params)
        w, fl = e.event_weights(gl["u"], prec=g.FP64)
        wo, flo = orc.weights(params, gl["u"])
    finally:
        params.regge.offshellFF = 2
    assert np.array_equal(fl & 1, gl["kin"])
    kin = gl["kin"] == 1
    assert np.array_equal(((fl >> 1) & 1)[kin], gl["fid"][kin])
    assert np.array_equal(fl, flo)
    assert _rel(w, gl["w"]).max() < TOL_FP64_REF
    assert _rel(w, wo).max() < TOL_FP64_ORC


def test_tree_weights_vs_oracle_large(gpu, params):
    """2^18 fresh points, weights and flags against the oracle."""
    import graniitti_gb300 as g
    e = _engine(params)
    u = e.uniforms(seed=99, n=1 << 18)
    w, fl = e.event_weights(u, prec=g.FP64)
    wo, flo = orc.weights(params, u, nthreads=16)
    assert np.array_equal(fl, flo)
    assert _rel(w, wo).max() < TOL_FP64_ORC
    # mixed precision does not change the tree level (FP64 Born)
    wm, _ = e.event_weights(u, prec=g.MIXED)
    assert _rel(wm, w).max() < 1e-13


def test_kinematics_vs_reference(gpu, params):
    gl = _load("c1_tune0_weights.npz")
    e = _engine(params)
    p4, ts, fl = e.event_kinematics(gl["u"])
    kin = gl["kin"] == 1
    scale = np.abs(gl["p4"]).max(axis=2, keepdims=True)
    assert (np.abs(p4 - gl["p4"])[kin] / scale[kin]).max() < 1e-12
    big = kin & (np.abs(gl["t1"]) > 1e-2)
    assert np.max(np.abs(ts[big, 0] - gl["t1"][big]) / np.abs(gl["t1"][big])) < 1e-8


def test_eikonal_tables_vs_reference(gpu, params_screened):
    g = _load("eikonal_nbt1024_nkt10000.npz")
    e = _engine(params_screened)
    e.eikonal_build(1024, 10000)
    xs = np.array(e.eikonal_xs())
    assert np.max(np.abs(xs / g["xs"] - 1)) < 1e-12
    mbt, msa = e.eikonal_tables(1024, 10000)
    for mine, ref in ((mbt, g["mbt"]), (msa, g["msa"])):
        assert np.max(np.abs(mine[:, 0] - ref[:, 0]) / np.maximum(1, np.abs(ref[:, 0]))) < 1e-13
        z, zr = mine[:, 1] + 1j * mine[:, 2], ref[:, 1] + 1j * ref[:, 2]
        assert np.max(np.abs(z - zr)) / np.max(np.abs(zr)) < 1e-12


@pytest.mark.parametrize("name", ["c2_screened_63x33_weights.npz", "c2_screened_15x12_weights.npz"])
def test_screened_weights_vs_reference(gpu, params_screened, name):
    import graniitti_gb300 as g
    gl = _load(name)
    t = _load("eikonal_nbt1024_nkt10000.npz")
    P = params_screened
    P.loop.n_kt, P.loop.n_phi = int(gl["loop_kt"]), int(gl["loop_phi"])
    P.loop.kt_max = float(gl["loop_ktmax"])
    e = _engine(P)
    e.eikonal_set(t["mbt"], t["msa"])  # the reference's own tables
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    assert np.array_equal(fl & 1, gl["kin"])
    assert _rel(w, gl["w"]).max() < 1e-9
    wm, _ = e.event_weights(gl["u"], prec=g.MIXED)
    Pb = type(P)()
    import ctypes
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = _engine(Pb).event_weights(gl["u"], prec=g.FP64)
    ok, rel = _mixed_ok(wm, w, wb)
    print("mixed vs fp64: max rel %.3e median %.3e" % (rel.max(), np.median(rel)))
    assert ok
    # GPU-built tables give the same weights
    e2 = _engine(P)
    e2.eikonal_build(1024, 10000)
    w2, _ = e2.event_weights(gl["u"], prec=g.FP64)
    assert _rel(w2, gl["w"]).max() < 1e-9


def test_screened_mixed_vs_oracle_c2_grid(gpu, params_screened):
    """Configuration of the benchmark: 63 x 33 loop intervals, kt <= 3 GeV,
    1024 b-points; FP32 compensated loop against the FP64 oracle."""
    import graniitti_gb300 as g
    P = params_screened
    P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = 63, 33, 3.0
    e = _engine(P)
    e.eikonal_build(1024, 10000)
    _, msa = e.eikonal_tables(1024, 10000)
    u = e.uniforms(seed=5, n=2048)
    wm, fm = e.event_weights(u, prec=g.MIXED)
    w64, f64 = e.event_weights(u, prec=g.FP64)
    wo, fo = orc.weights(P, u, msa=msa, nthreads=16)
    assert np.array_equal(fm, fo) and np.array_equal(f64, fo)
    assert _rel(w64, wo).max() < 1e-9
    import ctypes
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = _engine(Pb).event_weights(u, prec=g.FP64)
    ok, r = _mixed_ok(wm, wo, wb)
    print("mixed-precision screened weights: max rel %.3e, median %.3e, >1e-5: %d of %d" %
          (r.max(), np.median(r), int((r > 1e-5).sum()), r.size))
    assert ok


def _params_F(screened=False):
    from graniitti_gb300 import card
    from conftest import CARD, CARD_SCR
    return card.build_params(card.read_card(CARD_SCR if screened else CARD),
                             "PP[CON]<F> -> pi+ pi-")


def test_factorized_tree_vs_reference(gpu):
    import graniitti_gb300 as g
    gl = _load("f_tree_weights.npz")
    P = _params_F()
    e = _engine(P)
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    wo, flo = orc.weights(P, gl["u"])
    assert np.array_equal(fl & 1, gl["kin"])
    kin = gl["kin"] == 1
    assert np.array_equal(((fl >> 1) & 1)[kin], gl["fid"][kin])
    assert np.array_equal(fl, flo)
    assert _rel(w, gl["w"]).max() < TOL_FP64_REF
    assert _rel(w, wo).max() < TOL_FP64_ORC
    p4, ts, _ = e.event_kinematics(gl["u"])
    scale = np.abs(gl["p4"]).max(axis=2, keepdims=True)
    assert (np.abs(p4 - gl["p4"])[kin] / scale[kin]).max() < 1e-12


def test_factorized_screened_vs_reference(gpu):
    import graniitti_gb300 as g
    gl = _load("f_screened_15x12_weights.npz")
    t = _load("eikonal_nbt1024_nkt10000.npz")
    P = _params_F(True)
    e = _engine(P)
    e.eikonal_set(t["mbt"], t["msa"])
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    assert np.array_equal(fl & 1, gl["kin"])
    assert _rel(w, gl["w"]).max() < 1e-9
    wm, _ = e.event_weights(gl["u"], prec=g.MIXED)
    import ctypes
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = _engine(Pb).event_weights(gl["u"], prec=g.FP64)
    ok, rel = _mixed_ok(wm, w, wb)
    assert ok, rel.max()


def test_factorized_vegas_cross_section_vs_oracle_mc(gpu):
    """<F> and <C> describe the same process: their integrated cross sections
    agree within statistical errors (the reference's run_compare_PS check)."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi
    res = {}
    for cls in ("C", "F"):
        from graniitti_gb300 import card
        from conftest import CARD
        P = card.build_params(card.read_card(CARD), "PP[CON]<%s> -> pi+ pi-" % cls)
        e = g.Engine(P, 0)
        vp = _abi.VegasParams()
        vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, 1 << 20, 1.5
        vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 5e-4, 3, 0, 11
        res[cls] = e.vegas_integrate(vp)
    c, f = res["C"], res["F"]
    pull = (c.sigma - f.sigma) / np.hypot(c.sigma_err, f.sigma_err)
    print("sigma <C> %.5e +- %.1e, <F> %.5e +- %.1e, pull %.2f" %
          (c.sigma, c.sigma_err, f.sigma, f.sigma_err, pull))
    assert abs(pull) < 4


@pytest.mark.parametrize("name,proc", [
    ("t_tree_weights.npz", "PP[CONTENSOR]<C> -> pi+ pi-"),
    ("tf_tree_weights.npz", "PP[CONTENSOR]<F> -> pi+ pi-")])
def test_tensor_pomeron_tree_vs_reference(gpu, name, proc):
    import graniitti_gb300 as g
    from graniitti_gb300 import card
    from conftest import CARD
    gl = _load(name)
    P = card.build_params(card.read_card(CARD), proc)
    w, fl = _engine(P).event_weights(gl["u"], prec=g.FP64)
    wo, flo = orc.weights(P, gl["u"])
    assert np.array_equal(fl, flo) and np.array_equal(fl & 1, gl["kin"])
    assert _rel(w, gl["w"]).max() < TOL_FP64_REF
    assert _rel(w, wo).max() < TOL_FP64_ORC


def test_tensor_pomeron_screened_vs_reference(gpu):
    import ctypes
    import graniitti_gb300 as g
    from graniitti_gb300 import card
    from conftest import CARD_SCR
    gl = _load("t_screened_15x12_weights.npz")
    t = _load("eikonal_nbt1024_nkt10000.npz")
    P = card.build_params(card.read_card(CARD_SCR), "PP[CONTENSOR]<C> -> pi+ pi-")
    e = _engine(P)
    e.eikonal_set(t["mbt"], t["msa"])
    w, fl = e.event_weights(gl["u"], prec=g.FP64)
    assert np.array_equal(fl & 1, gl["kin"])
    assert _rel(w, gl["w"]).max() < 1e-9
    wm, _ = e.event_weights(gl["u"], prec=g.MIXED)
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = _engine(Pb).event_weights(gl["u"], prec=g.FP64)
    ok, rel = _mixed_ok(wm, w, wb)
    print("tensor mixed vs fp64: max rel %.3e" % rel.max())
    assert ok, rel.max()


@pytest.mark.parametrize("n", [2048, 2047])
def test_paired_loop_kernel_vs_fp64(gpu, params_screened, n):
    """The kt-loop with two events per thread (packed FP32x2 arithmetic) against the FP64
    loop, on the benchmark grid; odd n leaves the last thread with one event."""
    import ctypes
    import graniitti_gb300 as g
    P = params_screened
    P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = 63, 33, 3.0
    e = _engine(P)
    e.eikonal_build(1024, 10000)
    u = e.uniforms(seed=9, n=n)
    w64, f64 = e.event_weights(u, prec=g.FP64)
    e.set_tuning(loop_pair=0)
    w1, f1 = e.event_weights(u, prec=g.MIXED)
    e.set_tuning(loop_pair=1)
    w2, f2 = e.event_weights(u, prec=g.MIXED)
    e.set_tuning(loop_pair=2)  # the same kernel capped at 168 registers (3 blocks per SM)
    w3, f3 = e.event_weights(u, prec=g.MIXED)
    assert np.array_equal(f2, f64) and np.array_equal(f1, f64) and np.array_equal(f3, f64)
    Pb = type(P)()
    ctypes.memmove(ctypes.byref(Pb), ctypes.byref(P), ctypes.sizeof(P))
    Pb.screening = 0
    wb, _ = _engine(Pb).event_weights(u, prec=g.FP64)
    ok, r = _mixed_ok(w2, w64, wb)
    nz = w1 > 0
    d12 = np.abs(w2[nz] / w1[nz] - 1)
    print("paired loop: max rel vs FP64 %.3e (median %.3e); vs one-event kernel max %.3e"
          % (r.max(), np.median(r), d12.max()))
    assert ok and d12.max() < 1e-5
    assert np.max(np.abs(w3[nz] / w2[nz] - 1)) < 1e-6


def test_autotune_keeps_fastest_and_results(gpu, params_screened):
    import graniitti_gb300 as g
    P = params_screened
    P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = 63, 33, 3.0
    e = _engine(P)
    e.eikonal_build(1024, 10000)
    r = e.autotune(sample=1 << 16)
    ms = list(r.ms)[:r.n_candidates]
    print("autotune: %d candidates on %d events, ms %s, best pair=%d blocks=%d" %
          (r.n_candidates, r.sample_events, np.round(ms, 3), r.best.loop_pair,
           r.best.vegas_blocks))
    assert r.n_candidates == 8 and r.sample_events > 0
    k = int(np.argmin(ms))
    assert (r.best.loop_pair, r.best.vegas_blocks) == (r.cand[k].loop_pair, r.cand[k].vegas_blocks)
    t = e.tuning()
    assert (t.loop_pair, t.vegas_blocks) == (r.best.loop_pair, r.best.vegas_blocks)
    u = e.uniforms(seed=10, n=512)
    wm, _ = e.event_weights(u, prec=g.MIXED)
    w64, _ = e.event_weights(u, prec=g.FP64)
    nz = w64 > 0
    assert np.max(np.abs(wm[nz] / w64[nz] - 1)) < 1e-4


def test_autotune_on_the_vegas_loop_stage(gpu, params_screened):
    """With VEGAS initialised the autotuner times the loop stage of a full pass on the
    engine's grid; the passes after it integrate as before."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi
    P = params_screened
    e = _engine(P)
    e.eikonal_build(512, 2000)
    vp = _abi.VegasParams()
    vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, 1 << 17, 1.5
    vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, g.MIXED, 3
    e.vegas_init(vp)
    for it in range(2):
        e.vegas_iteration(mode=0, refine=True, iter_id=1 + it)
    grid = e.vegas_grid()
    r = e.autotune()
    ms = np.array(list(r.ms)[:r.n_candidates])
    stage = np.array(list(r.stage)[:r.n_candidates])
    print("VEGAS-stage autotune: %d candidates on %d listed events, ms %s, best stage A %d "
          "blocks, loop %d x %d" % (r.n_candidates, r.sample_events, np.round(ms, 3),
                                    r.best.born_blocks, r.best.loop_pair, r.best.vegas_blocks))
    # stage A: 4 grids; the record loop: 8 variant x grid candidates
    assert r.n_candidates == 12 and list(stage) == [0] * 4 + [1] * 8
    assert 0 < r.sample_events <= vp.ncall
    ka = int(np.argmin(ms[:4]))
    kl = 4 + int(np.argmin(ms[4:]))
    assert r.best.born_blocks == r.cand[ka].born_blocks
    assert (r.best.loop_pair, r.best.vegas_blocks) == (r.cand[kl].loop_pair, r.cand[kl].vegas_blocks)
    t = e.tuning()
    assert (t.born_blocks, t.loop_pair, t.vegas_blocks) == (r.best.born_blocks, r.best.loop_pair,
                                                            r.best.vegas_blocks)
    assert np.array_equal(e.vegas_grid(), grid)  # tuning does not refine
    res = [e.vegas_iteration(mode=1, refine=True, iter_id=10 + it) for it in range(2)]
    e.set_tuning(loop_pair=0)
    e.vegas_set_grid(grid)
    assert res[-1].sigma > 0 and res[-1].nan_count == 0


# The GPU engine in FP64 against the oracle restatement evaluated in long double (the
# reference's formulas and constants with its FP64 rounding removed; tests/golden/
# long_double_oracle.npz): 1e-10 relative on every point of every weight fixture, or, at a
# point where the reference's own FP64 weight is farther than that from the long-double value,
# no farther than the reference (a tensor-pomeron resonance point at a zero of the d-wave decay
# distribution, weight 1e-161 of the fixture's largest: engine 1.1e-10, reference 7.4e-10).
# The engine's light-cone formulation avoids the 4-vector cancellations that leave the
# reference's own FP64 weights up to 2.5e-9 from the same values.
LD_TOL = 1e-10


def _weight_fixtures():
    import sys
    sys.path.insert(0, GOLDEN)
    from fixture_meta import weight_fixtures
    return weight_fixtures()


@pytest.mark.parametrize("name", _weight_fixtures())
def test_fp64_engine_vs_long_double_oracle(gpu, name):
    import sys
    import graniitti_gb300 as g
    sys.path.insert(0, GOLDEN)
    from fixture_meta import fixture_params
    gl = _load(name)
    P, msa = fixture_params(name, gl)
    e = g.Engine(P, 0)
    if P.screening:
        t = _load("eikonal_nbt1024_nkt10000.npz")
        e.eikonal_set(t["mbt"], t["msa"])
    w, _ = e.event_weights(gl["u"], prec=g.FP64)
    wl = np.load(os.path.join(GOLDEN, "long_double_oracle.npz"))[name[:-4]]
    nz = wl > 0
    assert np.array_equal(w > 0, nz)
    r_eng = np.abs(w[nz] - wl[nz]) / wl[nz]
    both = nz & (gl["w"] > 0)
    r_ref = np.abs(gl["w"][both] - wl[both]) / wl[both]
    ok = r_eng < LD_TOL
    r_ref_all = np.zeros(nz.sum())  # no allowance where the reference has no weight
    r_ref_all[both[nz]] = r_ref
    beyond = ~ok
    print("%s: vs long double, engine FP64 max %.2e median %.2e; reference max %.2e; "
          "%d point(s) above %.0e, each nearer than the reference" %
          (name, r_eng.max(), np.median(r_eng), r_ref.max(), beyond.sum(), LD_TOL))
    assert np.all(ok | (r_eng <= r_ref_all)), r_eng.max()
    e.close()


def test_autotune_generic_loop_keeps_results(gpu):
    """A process outside record mode (tensor-pomeron f2(1270), screened): the tuner times the
    stage-A grid and the FP32 generic loop's grid; a VEGAS pass on the tuned grids gives the
    same integral bit for bit as on the default ones (every event is computed on its own and
    every sum has a fixed order)."""
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi, card
    from conftest import CARD_SCR
    c = card.read_card(CARD_SCR)
    c["PROCESSPARAM"]["RES"] = ["f2_1270"]
    P = card.build_params(c, "PP[RESTENSOR]<C> -> pi+ pi- @RES{f2_1270:1}")
    res = []
    for tune in (False, True):
        e = _engine(P)
        e.eikonal_build(512, 2000)
        vp = _abi.VegasParams()
        vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, 1 << 17, 1.5
        vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, g.MIXED, 3
        e.vegas_init(vp)
        for it in range(2):
            e.vegas_iteration(mode=0, refine=True, iter_id=1 + it)
        if tune:
            r = e.autotune()
            ms = np.array(list(r.ms)[:r.n_candidates])
            stage = list(r.stage)[:r.n_candidates]
            print("generic-loop autotune: ms %s, best stage A %d, generic loop %d blocks"
                  % (np.round(ms, 3), r.best.born_blocks, r.best.generic_blocks))
            assert stage == [0] * 4 + [2] * 3 and r.sample_events > 0
            kg = 4 + int(np.argmin(ms[4:]))
            assert r.best.generic_blocks == r.cand[kg].generic_blocks > 0
            assert e.tuning().generic_blocks == r.best.generic_blocks
        res.append(e.vegas_iteration(mode=1, refine=True, iter_id=10))
        e.close()
    assert res[0].I_this == res[1].I_this and res[0].refined == res[1].refined

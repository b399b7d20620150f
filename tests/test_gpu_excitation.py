"""Forward excitation (NSTARS = 1, 2; MProcess::SampleForwardMasses, src/MProcess.cc:1317-1365;
the inelastic vertex S3FINEL of MRegge::PomPomProtonVertex, src/MRegge.cc:637-644;
ForwardVolume, src/MProcess.cc:1399-1413) of the Regge pi+ pi- continuum on the GPU, against
the reference's weights of the same 10-dimensional points (its in-EventWeight draws served from
the lifted coordinates) and against the long-double oracle."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")
# the reference's own FP64 rounding on these points (forward legs as 4-vectors at pT <= 100 GeV,
# N* masses up to sqrt(0.05 s)) reaches 4e-8; the engine is within 1e-10 of the long-double
# oracle (tests/test_gpu_parity.py::test_fp64_engine_vs_long_double_oracle covers every fixture)
TOL_REF = 1e-7
TOL_LD = 1e-10


def _fixture(name):
    sys.path.insert(0, GOLDEN)
    from fixture_meta import fixture_params
    g = np.load(os.path.join(GOLDEN, name))
    P, msa = fixture_params(name, g)
    return g, P, msa


def _engine(P, msa):
    import graniitti_gb300 as gg
    e = gg.Engine(P, 0)
    if P.screening:
        t = np.load(os.path.join(GOLDEN, "eikonal_nbt1024_nkt10000.npz"))
        e.eikonal_set(t["mbt"], t["msa"])
    return e


@pytest.mark.parametrize("name", ["nstar1_c_tree_weights.npz", "nstar2_c_tree_weights.npz",
                                  "nstar1_f_tree_weights.npz", "nstar2_f_tree_weights.npz",
                                  "nstar1_c_screened_15x12_weights.npz"])
def test_excitation_weights_match_reference(gpu, name):
    import graniitti_gb300 as gg
    g, P, msa = _fixture(name)
    e = _engine(P, msa)
    assert e.dim == 10
    w, fl = e.event_weights(g["u"], prec=gg.FP64)
    assert np.array_equal(fl & 1, g["kin"])
    kin = g["kin"] == 1
    assert np.array_equal(((fl >> 1) & 1)[kin], g["fid"][kin])
    nz = g["w"] > 0
    assert np.array_equal(w > 0, nz) and nz.sum() > 50
    r = np.abs(w[nz] - g["w"][nz]) / g["w"][nz]
    wl = np.load(os.path.join(GOLDEN, "long_double_oracle.npz"))[name[:-4]]
    rl = np.abs(w[nz] - wl[nz]) / wl[nz]
    print("%s: %d points with W > 0; engine vs reference max %.2e, vs long double max %.2e" %
          (name, nz.sum(), r.max(), rl.max()))
    assert r.max() < TOL_REF and rl.max() < TOL_LD
    # the forward legs' 4-momenta (pfinal[1], pfinal[2]: the excited masses)
    p4, _, kflags = e.event_kinematics(g["u"])
    ok = kin & ((kflags & 1) == 1)
    for k in (0, 1):
        d = np.abs(p4[ok, k] - g["p4"][ok, k]).max(axis=1) / np.abs(g["p4"][ok, k]).max(axis=1)
        assert d.max() < 1e-10, d.max()
    e.close()


def test_excitation_fp32_loop_vs_fp64(gpu):
    """Screened single excitation in MIXED precision against FP64 on 2^14 seeded points: with
    an excited leg the Regge exponents alpha(t) ln s reach 10^2 and more, beyond what the FP32
    loop resolves to 1e-5, so MIXED hands these events to the FP64 loop; without the
    refinement the FP32 loop (per-leg masses, closed-form light-cone closure, event scale)
    still gives their weights to ~1e-4."""
    import graniitti_gb300 as gg
    import philox_np
    g, P, msa = _fixture("nstar1_c_screened_15x12_weights.npz")
    e = _engine(P, msa)
    u = philox_np.uniforms(93, 1 << 14, 10)
    w64, fl = e.event_weights(u, prec=gg.FP64)
    wm, flm = e.event_weights(u, prec=gg.MIXED)
    assert np.array_equal(fl, flm)
    nz = w64 > 0
    r = np.abs(wm[nz] - w64[nz]) / w64[nz]
    print("screened excitation: MIXED vs FP64 over %d points: max %.2e, median %.2e" %
          (nz.sum(), r.max(), np.median(r)))
    assert nz.sum() > 1000 and r.max() < 1e-5
    e.set_tuning(fp64_refine=0)
    w32, _ = e.event_weights(u, prec=gg.MIXED)
    big = nz & (w64 > 1e-30 * w64.max())  # the weights that the FP32 range holds
    r32 = np.abs(w32[big] - w64[big]) / w64[big]
    print("   FP32 loop alone over %d points: median %.2e, p99 %.2e" %
          (big.sum(), np.median(r32), np.quantile(r32, 0.99)))
    assert np.median(r32) < 1e-5
    e.close()


def test_excitation_vegas_matches_flat_oracle_mean(gpu):
    """sigma(NSTARS = 1, <C>, tree level) from GPU VEGAS against the oracle's flat Monte Carlo
    mean of the same integrand (2^18 seeded points, 16 threads)."""
    import graniitti_gb300 as gg
    from graniitti_gb300 import _abi
    from oracle import oracle_api as orc
    import philox_np
    g, P, msa = _fixture("nstar1_c_tree_weights.npz")
    e = _engine(P, msa)
    vp = _abi.VegasParams()
    vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, 1 << 21, 1.5
    vp.chi2max, vp.precision, vp.burnin_iter, vp.prec, vp.seed = 10.0, 1e-3, 3, gg.FP64, 5
    e.vegas_init(vp)
    for it in range(6):
        e.vegas_iteration(mode=0, refine=True, iter_id=it)
    e.vegas_clear()
    r = None
    for it in range(4):
        r = e.vegas_iteration(mode=1, refine=True, iter_id=10 + it)
    u = philox_np.uniforms(94, 1 << 18, 10)
    wo, _ = orc.weights(P, u, nthreads=16)
    mean, err = wo.mean(), wo.std() / np.sqrt(len(wo))
    pull = (r.sigma - mean) / np.hypot(r.sigma_err, err)
    print("NSTARS=1 sigma: GPU VEGAS %.5e +- %.1e b, oracle flat mean %.5e +- %.1e b, pull %.2f"
          % (r.sigma, r.sigma_err, mean, err, pull))
    assert abs(pull) < 4
    e.close()

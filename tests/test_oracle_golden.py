"""The CPU oracle against golden vectors produced by the unmodified reference.

These pins are what make the oracle trustworthy as the checker of the GPU path.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import oracle_api as orc

# Reference and oracle solve the forward-leg kinematics with different (equivalent)
# formulas; the reference's own rounding noise reaches ~1e-10 on weights.
W_TOL = 5e-10


def _load(name):
    return np.load(os.path.join(GOLDEN, name))


def _check_weights(w, fl, g, tol=W_TOL):
    assert np.array_equal(fl & 1, g["kin"]), "kinematics flags differ"
    kin = g["kin"] == 1
    assert np.array_equal(((fl >> 1) & 1)[kin], g["fid"][kin]), "fiducial flags differ"
    wr = g["w"]
    assert np.array_equal(w > 0, wr > 0)
    nz = wr > 0
    rel = np.abs(w[nz] - wr[nz]) / wr[nz]
    assert rel.max() < tol, rel.max()
    return rel


@pytest.mark.parametrize("name,ff", [("c1_tune0_weights.npz", 2), ("c1_expff_weights.npz", 0),
                                     ("c1_orearff_weights.npz", 1), ("c1_edge_weights.npz", 2)])
def test_tree_weights(params, name, ff):
    g = _load(name)
    params.regge.offshellFF = ff
    try:
        w, fl, rec = orc.weights(params, g["u"], with_rec=True)
    finally:
        params.regge.offshellFF = 2
    _check_weights(w, fl, g)
    kin = g["kin"] == 1
    # forward legs and central particles (px, py, pz, E)
    p4 = rec[:, 3:19].reshape(-1, 4, 4)
    scale = np.abs(g["p4"]).max(axis=2, keepdims=True)
    assert (np.abs(p4 - g["p4"])[kin] / scale[kin]).max() < 1e-12
    # invariants: m2 everywhere, t1/t2 where |t| is not cancellation-limited in the reference
    assert np.max(np.abs(rec[kin, 2] - g["m2"][kin]) / g["m2"][kin]) < 1e-10
    big = kin & (np.abs(g["t1"]) > 1e-2)
    assert np.max(np.abs(rec[big, 0] - g["t1"][big]) / np.abs(g["t1"][big])) < 1e-8


def test_eikonal_tables_and_xs(params_screened):
    g = _load("eikonal_nbt1024_nkt10000.npz")
    mbt, msa, xs = orc.eikonal(params_screened, 1024, 10000, nthreads=8)
    assert np.max(np.abs(xs / g["xs"] - 1)) < 1e-12
    for mine, ref in ((mbt, g["mbt"]), (msa, g["msa"])):
        assert np.max(np.abs(mine[:, 0] - ref[:, 0]) / np.maximum(1, np.abs(ref[:, 0]))) < 1e-13
        z, zr = mine[:, 1] + 1j * mine[:, 2], ref[:, 1] + 1j * ref[:, 2]
        assert np.max(np.abs(z - zr)) / np.max(np.abs(zr)) < 1e-12


def test_eikonal_xs_default_numerics(params_screened):
    """Total / elastic / inelastic cross sections at 13 TeV, TUNE0, 10000 x 10000."""
    g = _load("eikonal_default_xs.npz")
    _, _, xs = orc.eikonal(params_screened, 10000, 10000, nthreads=8, with_msa=False)
    assert np.max(np.abs(xs / g["xs"] - 1)) < 1e-12
    # published-style values in mb
    assert abs(xs[0] * 1e3 - 105.08) < 0.01 and abs(xs[1] * 1e3 - 27.00) < 0.01


@pytest.mark.parametrize("name", ["c2_screened_63x33_weights.npz", "c2_screened_15x12_weights.npz"])
def test_screened_weights(params_screened, name):
    g = _load(name)
    t = _load("eikonal_nbt1024_nkt10000.npz")
    P = params_screened
    P.loop.n_kt, P.loop.n_phi = int(g["loop_kt"]), int(g["loop_phi"])
    P.loop.kt_max = float(g["loop_ktmax"])
    w, fl = orc.weights(P, g["u"], msa=t["msa"], nthreads=4)
    _check_weights(w, fl, g, tol=1e-9)


def test_bessel_j0_published_values():
    # A&S Table 9.1 values of J0 (accuracy of the published approximation ~1e-8)
    for x, v in ((0.0, 1.0), (1.0, 0.7651976866), (2.0, 0.2238907791), (5.0, -0.1775967713),
                 (10.0, -0.2459357645), (20.0, 0.1670246643)):
        assert abs(orc.bessel_j0(x) - v) < 2e-8


def test_vegas_grid_uniform_and_refine():
    x = orc.vegas_grid_init(128, 8)
    assert np.allclose(x, (np.arange(1, 129) / 128.0)[:, None], rtol=0, atol=1e-15)
    # a flat f^2 histogram leaves the uniform grid unchanged
    x2 = orc.vegas_refine(x, np.ones((128, 8)))
    assert np.allclose(x2, x, atol=1e-12)
    # a peaked histogram concentrates bins where f^2 is large
    f2 = np.ones((128, 8))
    f2[:16, 0] = 1e4
    x3 = orc.vegas_refine(x, f2)
    assert x3[63, 0] < x[63, 0] and np.all(np.diff(x3[:, 0]) > 0)
    assert np.allclose(x3[:, 1:], x[:, 1:], atol=1e-12)


def _params_F(screened=False):
    from graniitti_gb300 import card
    from conftest import CARD, CARD_SCR
    return card.build_params(card.read_card(CARD_SCR if screened else CARD),
                             "PP[CON]<F> -> pi+ pi-")


def test_factorized_tree_weights():
    g = _load("f_tree_weights.npz")
    w, fl, rec = orc.weights(_params_F(), g["u"], with_rec=True)
    _check_weights(w, fl, g)
    kin = g["kin"] == 1
    p4 = rec[:, 3:19].reshape(-1, 4, 4)
    scale = np.abs(g["p4"]).max(axis=2, keepdims=True)
    assert (np.abs(p4 - g["p4"])[kin] / scale[kin]).max() < 1e-12


def test_factorized_screened_weights():
    g = _load("f_screened_15x12_weights.npz")
    t = _load("eikonal_nbt1024_nkt10000.npz")
    w, fl = orc.weights(_params_F(True), g["u"], msa=t["msa"], nthreads=4)
    _check_weights(w, fl, g, tol=1e-9)


def _params(proc, screened=False):
    from graniitti_gb300 import card
    from conftest import CARD, CARD_SCR
    return card.build_params(card.read_card(CARD_SCR if screened else CARD), proc)


@pytest.mark.parametrize("name,proc", [
    ("t_tree_weights.npz", "PP[CONTENSOR]<C> -> pi+ pi-"),
    ("tf_tree_weights.npz", "PP[CONTENSOR]<F> -> pi+ pi-")])
def test_tensor_pomeron_tree_weights(name, proc):
    g = _load(name)
    w, fl = orc.weights(_params(proc), g["u"])
    _check_weights(w, fl, g)


def test_tensor_pomeron_screened_weights():
    g = _load("t_screened_15x12_weights.npz")
    t = _load("eikonal_nbt1024_nkt10000.npz")
    w, fl = orc.weights(_params("PP[CONTENSOR]<C> -> pi+ pi-", True), g["u"], msa=t["msa"],
                        nthreads=4)
    _check_weights(w, fl, g, tol=1e-9)


# Tensor-pomeron resonances (PROC_11, MTensorPomeron::ME3): the fixtures carry their card and
# process string (with the @RES / @R commands the reference parsed).
def _params_res(g):
    from graniitti_gb300 import card
    return card.build_params(card.read_card(os.path.join(GOLDEN, "cards", str(g["card"]))),
                             str(g["proc"]))


# The tensor amplitude has zeros in the decay angle; near them the reference's Cartesian
# contractions of 13 TeV 4-vectors (and the oracle's) lose relative precision, which puts
# a few points at 1e-9 while the median stays at 2e-11.
RES_TOL = 5e-9


@pytest.mark.parametrize("name", ["rf_tree_weights.npz", "rf_mix_tree_weights.npz",
                                  "rf_kk_tree_weights.npz", "rc_tree_weights.npz",
                                  "rf_f2_1525_tree_weights.npz"] +
                         ["rf_s%d_tree_weights.npz" % j for j in range(1, 7)] +
                         ["rcf_tree_weights.npz", "rcc_tree_weights.npz", "rck_tree_weights.npz"] +
                         ["gr_tree_weights.npz", "grc_tree_weights.npz", "grc_hx_tree_weights.npz",
                          "grc_cm_jz_tree_weights.npz", "grc_nogen_tree_weights.npz",
                          "grc_kk_tree_weights.npz", "grc_c_tree_weights.npz"])
def test_tensor_resonance_tree_weights(lib_built, name):
    g = _load(name)
    w, fl = orc.weights(_params_res(g), g["u"])
    rel = _check_weights(w, fl, g, tol=RES_TOL)
    assert np.median(rel) < 1e-10


@pytest.mark.parametrize("name", ["rf_screened_15x12_weights.npz",
                                  "rcf_screened_15x12_weights.npz",
                                  "grc_screened_15x12_weights.npz"])
def test_tensor_resonance_screened_weights(lib_built, name):
    g = _load(name)
    t = _load("eikonal_nbt1024_nkt10000.npz")
    w, fl = orc.weights(_params_res(g), g["u"], msa=t["msa"], nthreads=4)
    _check_weights(w, fl, g, tol=1e-9)


# Two-body cascades of vector-meson pairs: tensor-pomeron 2xV (MTensorPomeron::ME4 :808-888)
# and the Regge continuum, with the final-state daughters; <F> (14 dimensions, or 12 with
# @OFFSHELL:0) and the continuum class <C> (MContinuum::BNRandomKin / BNBuildKin with
# ConstructDecayKinematics: 12 dimensions with @OFFSHELL:0, 14 with the Breit-Wigner masses).
@pytest.mark.parametrize("name", ["rr_tree_weights.npz", "rr_regge_tree_weights.npz",
                                  "ff_tree_weights.npz", "rr_screened_15x12_weights.npz",
                                  "rrc_tree_weights.npz", "rrc_regge_tree_weights.npz",
                                  "rrc14_tree_weights.npz", "rrf12_tree_weights.npz",
                                  "rrc_screened_15x12_weights.npz"])
def test_vector_pair_cascade_weights(name):
    g = _load(name)
    P = _params_res(g)
    assert P.n_decay == 2 and P.central_spin == 1
    assert g["u"].shape[1] == (12 if "@OFFSHELL:0" in str(g["proc"]) else 14)
    msa = _load("eikonal_nbt1024_nkt10000.npz")["msa"] if P.screening else None
    w, fl, rec = orc.weights(P, g["u"], msa=msa, nthreads=4, with_rec=True)
    _check_weights(w, fl, g, tol=W_TOL)
    kin = g["kin"] == 1
    leaves = rec[:, 19:35].reshape(-1, 4, 4)
    scale = np.abs(g["leaves"]).max(axis=2, keepdims=True)
    assert (np.abs(leaves - g["leaves"])[kin] / scale[kin]).max() < 1e-12


@pytest.mark.parametrize("name", ["f4_tree_weights.npz", "f4_kk_tree_weights.npz",
                                  "f4_screened_weights.npz", "c4_tree_weights.npz",
                                  "c4_screened_weights.npz", "f6_tree_weights.npz",
                                  "c6_tree_weights.npz", "f6_screened_weights.npz",
                                  "c6_screened_weights.npz"])
def test_n_body_continuum_weights(name):
    """PP[CON]<F|C> -> 4 or 6 bodies (MRegge::ME6 / ME8 with the weighted N-body phase space,
    or the continuum class's 14- or 20-dimensional phase space)."""
    g = _load(name)
    P = _params_res(g)
    assert P.n_central == (6 if name[1] == "6" else 4)
    msa = _load("eikonal_nbt1024_nkt10000.npz")["msa"] if P.screening else None
    w, fl, rec = orc.weights(P, g["u"], msa=msa, nthreads=4, with_rec=True)
    _check_weights(w, fl, g, tol=W_TOL)
    kin = g["kin"] == 1
    cen = rec[:, 19:35].reshape(-1, 4, 4)  # the first four central particles
    ref = g["leaves"][:, :4]
    scale = np.abs(ref).max(axis=2, keepdims=True)
    assert (np.abs(cen - ref)[kin] / scale[kin]).max() < 1e-12


def _np_rest(X, p):
    """p (n, 4: px, py, pz, E) boosted to the rest frame of X (n, 4)."""
    m = np.sqrt(X[:, 3] ** 2 - (X[:, :3] ** 2).sum(1))
    b = X[:, :3] / X[:, 3:4]
    g = X[:, 3] / m
    bp = (b * p[:, :3]).sum(1)
    b2 = (b * b).sum(1)
    k = np.where(b2 > 0, (g - 1) * bp / np.where(b2 > 0, b2, 1), 0.0) - g * p[:, 3]
    return np.column_stack([p[:, :3] + k[:, None] * b, g * (p[:, 3] - bp)])


def test_histogram_observables_from_reference_kinematics(params):
    """orc_observables against a numpy restatement of the reference's observables
    (MUserHistograms::FillHistograms, src/MUserHistograms.cc:60-125; frames of
    kinematics::LorentzFrame, MKinematics.h:952-1011) evaluated on the reference's own
    4-momenta of the same points."""
    from graniitti_gb300 import _abi
    g = _load("c1_tune0_weights.npz")
    kin = g["kin"] == 1
    obs, ok = orc.observables(params, g["u"])
    assert np.array_equal(ok, kin)
    p4 = g["p4"][kin]  # forward leg 1, forward leg 2, central 3, central 4
    o = obs[kin]
    X = p4[:, 2] + p4[:, 3]
    n = len(X)
    ref = {}
    ref["M"] = np.sqrt(X[:, 3] ** 2 - (X[:, :3] ** 2).sum(1))
    ref["Y"] = 0.5 * np.log((X[:, 3] + X[:, 2]) / (X[:, 3] - X[:, 2]))
    ref["PT"] = np.hypot(X[:, 0], X[:, 1])
    d = np.arctan2(p4[:, 0, 1], p4[:, 0, 0]) - np.arctan2(p4[:, 1, 1], p4[:, 1, 0])
    d = np.where(d >= np.pi, d - 2 * np.pi, d)
    d = np.where(d < -np.pi, d + 2 * np.pi, d)
    ref["DPHI_PP"] = np.abs(d)
    ref["PT1"] = np.hypot(p4[:, 0, 0], p4[:, 0, 1])
    for k, j in (("RAP3", 2), ("RAP4", 3)):
        ref[k] = 0.5 * np.log((p4[:, j, 3] + p4[:, j, 2]) / (p4[:, j, 3] - p4[:, j, 2]))
    ref["M0"] = np.sqrt(np.maximum(p4[:, 2, 3] ** 2 - (p4[:, 2, :3] ** 2).sum(1), 0))
    E = 0.5 * params.sqrt_s
    pz = np.sqrt(E * E - params.m_beam ** 2)
    b1 = _np_rest(X, np.tile([0, 0, pz, E], (n, 1)))[:, :3]
    b2 = _np_rest(X, np.tile([0, 0, -pz, E], (n, 1)))[:, :3]
    p = _np_rest(X, p4[:, 2])[:, :3]

    def unit(v):
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    u1, u2 = unit(b1), unit(b2)
    yax = unit(np.cross(u1, u2))
    frames = {"CS": unit(u1 - u2), "HX": unit(-(b1 + b2)), "AH": unit(u1 + u2), "PG": u2}
    for name, z in frames.items():
        x = unit(np.cross(yax, z))
        q = np.column_stack([(p * x).sum(1), (p * yax).sum(1), (p * z).sum(1)])
        ref["COSTH_" + name] = q[:, 2] / np.linalg.norm(q, axis=1)
        ref["PHI_" + name] = np.arctan2(q[:, 1], q[:, 0])
    ref["COSTH_CM"] = p[:, 2] / np.linalg.norm(p, axis=1)
    ref["PHI_CM"] = np.arctan2(p[:, 1], p[:, 0])
    lab = p4[:, 2, :3]
    ref["COSTH_LA"] = lab[:, 2] / np.linalg.norm(lab, axis=1)
    ref["PHI_LA"] = np.arctan2(lab[:, 1], lab[:, 0])
    assert set(ref) == set(_abi.OBS)
    # the anti-helicity axis is the sum of two nearly opposite unit vectors: its direction
    # carries the rounding of both divided by their sum's length
    ah_cond = 1.0 / np.linalg.norm(u1 + u2, axis=1)
    for k, v in ref.items():
        mine = o[:, _abi.OBS.index(k)]
        if k.startswith("PHI"):  # compare angles on the circle
            diff = np.abs(np.angle(np.exp(1j * (mine - v))))
        else:
            diff = np.abs(mine - v) / np.maximum(1.0, np.abs(v))
        if k.endswith("_AH"):
            diff = diff / ah_cond
        assert diff.max() < 1e-8, (k, diff.max())


# Forward excitation: the reference's own FP64 weights carry up to 4e-8 of rounding here (its
# 4-vector forward legs at pT <= 100 GeV and N* masses up to sqrt(0.05 s); both it and the FP64
# oracle are within that of the long-double oracle, see test_fp64_evaluations_vs_long_double).
EXC_TOL = 1e-7


@pytest.mark.parametrize("name", ["nstar1_c_tree_weights.npz", "nstar2_c_tree_weights.npz",
                                  "nstar1_f_tree_weights.npz", "nstar2_f_tree_weights.npz",
                                  "nstar1_c_screened_15x12_weights.npz"])
def test_forward_excitation_weights(name):
    """NSTARS = 1, 2 (MProcess::SampleForwardMasses, PomPomProtonVertex with S3FINEL,
    ForwardVolume): the oracle against the reference's weights of the same 10-dimensional
    points, both classes, tree level and screened."""
    import sys
    sys.path.insert(0, GOLDEN)
    from fixture_meta import fixture_params
    g = _load(name)
    P, msa = fixture_params(name, g)
    assert P.excitation in (1, 2) and g["u"].shape[1] == 10
    w, fl = orc.weights(P, g["u"], msa=msa, nthreads=8)
    rel = _check_weights(w, fl, g, tol=EXC_TOL)
    print("%s: oracle vs reference max rel %.2e median %.2e" % (name, rel.max(), np.median(rel)))


@pytest.mark.parametrize("name", ["veto_c_weights.npz", "veto_rr_weights.npz",
                                  "veto_f4_weights.npz"])
def test_veto_cuts(name):
    """Veto domains on the final-state leaves: flags and weights as the reference's."""
    g = _load(name)
    P = _params_res(g)
    assert P.veto_active == 1 and P.n_veto == 2
    w, fl = orc.weights(P, g["u"], nthreads=4)
    _check_weights(w, fl, g, tol=W_TOL)
    kin = g["kin"] == 1
    assert np.array_equal(((fl >> 2) & 1)[kin], g["veto"][kin])
    assert (g["veto"][kin] == 0).sum() > 100


# The restatement in long double arithmetic (oracle/_build/liborc_ld.so): the same formulas
# and constants as the reference with 11 more significand bits (x86), i.e. the reference's own
# value with its FP64 rounding removed. tests/golden/long_double_oracle.npz holds its weights
# for every weight fixture (make_golden.py --only ld).
def test_long_double_oracle_reproduces_stored_weights():
    import sys
    sys.path.insert(0, GOLDEN)
    from fixture_meta import fixture_params
    ld = np.load(os.path.join(GOLDEN, "long_double_oracle.npz"))
    for name in ("c1_tune0_weights.npz", "rc_tree_weights.npz", "rrc_tree_weights.npz",
                 "c2_screened_63x33_weights.npz"):
        g = _load(name)
        P, msa = fixture_params(name, g)
        w, _ = orc.weights(P, g["u"], msa=msa, nthreads=8, long_double=True)
        wl = ld[name[:-4]]
        nz = wl > 0
        assert np.array_equal(w > 0, nz)
        assert np.max(np.abs(w[nz] - wl[nz]) / wl[nz]) < 1e-13


def test_fp64_evaluations_vs_long_double():
    """How far FP64 evaluations of the reference's formulas sit from their long-double value:
    the reference itself and the FP64 oracle both carry up to ~2.5e-9 relative rounding on
    fixtures where 13 TeV 4-vector products cancel (tensor resonances in <C>), typically
    1e-10, and up to 4e-8 with excited forward legs (N* 4-vectors of mass up to sqrt(0.05 s),
    forward pT up to 100 GeV); the tests of the GPU engine compare it with the long-double
    weights."""
    import sys
    sys.path.insert(0, GOLDEN)
    from fixture_meta import fixture_params, weight_fixtures
    ld = np.load(os.path.join(GOLDEN, "long_double_oracle.npz"))
    worst_ref = worst_orc = worst_exc = 0.0
    for name in weight_fixtures():
        g = _load(name)
        if g["u"].shape[0] > 1024 or "loop_kt" in g or "n_bt" in g:
            continue  # the large and the screened fixtures: covered by the GPU comparison
        P, msa = fixture_params(name, g)
        w, _ = orc.weights(P, g["u"], msa=msa, nthreads=8)
        wl = ld[name[:-4]]
        nz = (wl > 0) & (g["w"] > 0)
        r_ref = np.max(np.abs(g["w"][nz] - wl[nz]) / wl[nz])
        r_orc = np.max(np.abs(w[nz] - wl[nz]) / wl[nz])
        if P.excitation:
            worst_exc = max(worst_exc, r_ref, r_orc)
        else:
            worst_ref = max(worst_ref, r_ref)
            worst_orc = max(worst_orc, r_orc)
    print("vs long double: reference %.2e, FP64 oracle %.2e; with excitation %.2e" %
          (worst_ref, worst_orc, worst_exc))
    assert worst_ref < 3e-9 and worst_orc < 3e-9 and worst_exc < 1e-7

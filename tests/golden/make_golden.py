"""Generate the golden fixtures under tests/golden/ from the UNMODIFIED reference.

Runs here (x86 container with the reference sources); the fixtures travel, the
reference does not. Steps:
  1. build the reference driver: make -C oracle/refbuild (oracle/_ref/bin/grn_ref)
  2. draw Philox4x32-10 points (tests/philox_np.py), feed them to the reference's
     MProcess::EventWeight, store points + weights + flags + kinematics
  3. build the eikonal tables with the reference's MEikonal::S3Constructor
  4. run the reference VEGAS integration for the cross section

Usage: python tests/golden/make_golden.py [--ref <reference source tree>]
                                          [--only resonances|cascades|rescon|regge_res|
                                                  nbody|nbody_c|nbody6|veto|ccascades|
                                                  excitation|ld]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.abspath(os.path.join(HERE, "..", ".."))
sys.path.insert(0, os.path.join(REPO, "tests"))
import philox_np  # noqa: E402

REF_BIN = os.path.join(REPO, "oracle", "_ref", "bin", "grn_ref")
CARD = os.path.join(HERE, "cards", "pp_con_pipi.json")
CARD_SCR = os.path.join(HERE, "cards", "pp_con_pipi_screened.json")
PROC = "PP[CON]<C> -> pi+ pi-"
# point and weight files exchanged with the reference driver (a fresh temporary folder)
TMP = tempfile.mkdtemp(prefix="grn_golden_")
# the reference source tree: $GRANIITTI_REFERENCE, else a "reference" folder beside the repo
REF_DEFAULT = os.environ.get("GRANIITTI_REFERENCE",
                             os.path.join(os.path.dirname(REPO), "reference"))


def run_weights(card, u, extra=(), proc=PROC, dim=None, leaves=0):
    """Reference weights of points u (n x 8). For <F> the process dimension is 6 and
    the decay angles are served from u[:, 6:8] through the RNG replay (the two pion
    off-shell mass draws, numerically inert at width 2.5e-17 GeV, take 0.5)."""
    os.makedirs(TMP, exist_ok=True)
    uf = os.path.join(TMP, "u.bin")
    wf = os.path.join(TMP, "w.bin")
    u.astype(np.float64).tofile(uf)
    dim = dim or u.shape[1]
    cmd = [REF_BIN, "weights", card, proc, uf, str(dim), wf] + list(extra)
    if dim != u.shape[1]:
        cmd += ["--stride", str(u.shape[1])]
    if leaves:
        cmd += ["--leaves", str(leaves)]
    subprocess.run(cmd, check=True, capture_output=True)
    r = np.fromfile(wf).reshape(-1, 24 + 4 * leaves)
    out = dict(w=r[:, 0], kin=r[:, 1].astype(np.uint8), fid=r[:, 2].astype(np.uint8),
               veto=r[:, 3].astype(np.uint8), amp=r[:, 4].astype(np.uint8), t1=r[:, 5],
               t2=r[:, 6], m2=r[:, 7], p4=r[:, 8:24].reshape(-1, 4, 4))
    if leaves:
        out["leaves"] = r[:, 24:].reshape(-1, leaves, 4)
    return out


def save(name, **arrays):
    np.savez_compressed(os.path.join(HERE, name), **arrays)
    print("wrote", name)


CARD_RES = os.path.join(HERE, "cards", "pp_res_pipi.json")
CARD_RES_SCR = os.path.join(HERE, "cards", "pp_res_pipi_screened.json")


def resonance_fixtures():
    """Tensor-pomeron resonances (PROC_11, MTensorPomeron::ME3): f2(1270) alone, four
    resonances with an @R override, the K+ K- decay (f0(980) below threshold), the <C>
    class, and the screened amplitude."""
    REPLAY_F = ["--replay", "h,h,6,7"]
    cases = [
        ("rf_tree_weights.npz", 61, 2048, CARD_RES, "PP[RESTENSOR]<F> -> pi+ pi-", REPLAY_F, 6),
        ("rf_mix_tree_weights.npz", 62, 1024, CARD_RES,
         "PP[RESTENSOR]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1, f0_1500:1, f0_1710:1} "
         "@R[f2_1270]{M:1.3, W:0.2, g0:1.5}", REPLAY_F, 6),
        ("rf_kk_tree_weights.npz", 63, 512, CARD_RES,
         "PP[RESTENSOR]<F> -> K+ K- @RES{f0_980:1, f2_1270:1}", REPLAY_F, 6),
        ("rc_tree_weights.npz", 64, 1024, CARD_RES,
         "PP[RESTENSOR]<C> -> pi+ pi- @RES{f0_980:1, f2_1270:1}", [], 8),
    ]
    for name, seed, n, card, proc, extra, dim in cases:
        u = philox_np.uniforms(seed, n, 8)
        r = run_weights(card, u, extra, proc=proc, dim=dim)
        save(name, seed=seed, u=u, card=os.path.basename(card), proc=proc, **r)
    # The J = 2 coupling structures one at a time (g_j = 1, the others 0), and TUNE0's
    # f2(1525) (structure 1), at forward pT >= 0.05 GeV (u[0], u[1] >= 0.86): structures 1 and
    # 4 vanish as the forward pT go to zero, and the reference's Cartesian contractions leave
    # only rounding noise there.
    for j in range(1, 7):
        g = ", ".join("g%d:%s" % (i, "1.0" if i == j else "0.0") for i in range(7))
        proc = "PP[RESTENSOR]<F> -> pi+ pi- @RES{f2_1270:1} @R[f2_1270]{%s}" % g
        u = philox_np.uniforms(70 + j, 256, 8)
        u[:, :2] = 0.86 + 0.14 * u[:, :2]
        r = run_weights(CARD_RES, u, REPLAY_F, proc=proc, dim=6)
        save("rf_s%d_tree_weights.npz" % j, seed=70 + j, u=u, card=os.path.basename(CARD_RES),
             proc=proc, **r)
    proc = "PP[RESTENSOR]<F> -> pi+ pi- @RES{f2_1525:1, f2_1270:1}"
    u = philox_np.uniforms(77, 256, 8)
    u[:, :2] = 0.86 + 0.14 * u[:, :2]
    r = run_weights(CARD_RES, u, REPLAY_F, proc=proc, dim=6)
    save("rf_f2_1525_tree_weights.npz", seed=77, u=u, card=os.path.basename(CARD_RES), proc=proc,
         **r)
    proc = "PP[RESTENSOR]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1}"
    u = philox_np.uniforms(65, 96, 8)
    r = run_weights(CARD_RES_SCR, u, REPLAY_F + ["--nbt", "1024", "--nkt2", "10000"], proc=proc,
                    dim=6)
    save("rf_screened_15x12_weights.npz", seed=65, u=u, card=os.path.basename(CARD_RES_SCR),
         proc=proc, n_bt=1024, n_kt2=10000, loop_kt=15, loop_phi=12, loop_ktmax=1.75, **r)
    # VEGAS cross section of the f2(1270) card (reference ranlux48 points, 8 threads).
    out = subprocess.run([REF_BIN, "vegas", CARD_RES, "PP[RESTENSOR]<F> -> pi+ pi-", "--cores",
                          "8"], check=True, capture_output=True, text=True).stdout
    write_sigma("rf_vegas_sigma.json", out, "PP[RESTENSOR]<F> -> pi+ pi-",
                os.path.basename(CARD_RES))


def rescon_fixtures():
    """Tensor-pomeron resonances + 2xS continuum (PROC_14, RES+CONTENSOR): the coherent sum
    exercises the relative phase of the two amplitudes (<F> and <C>, K+ K-, screened)."""
    REPLAY_F = ["--replay", "h,h,6,7"]
    cases = [
        ("rcf_tree_weights.npz", 91, 1024, CARD_RES,
         "PP[RES+CONTENSOR]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1}", REPLAY_F, 6),
        ("rcc_tree_weights.npz", 92, 1024, CARD_RES,
         "PP[RES+CONTENSOR]<C> -> pi+ pi- @RES{f0_980:1, f2_1270:1, f0_1500:1}", [], 8),
        ("rck_tree_weights.npz", 93, 512, CARD_RES,
         "PP[RES+CONTENSOR]<F> -> K+ K- @RES{f0_980:1, f2_1270:1, f2_1525:1}", REPLAY_F, 6),
    ]
    for name, seed, n, card, proc, extra, dim in cases:
        u = philox_np.uniforms(seed, n, 8)
        r = run_weights(card, u, extra, proc=proc, dim=dim)
        save(name, seed=seed, u=u, card=os.path.basename(card), proc=proc, **r)
    proc = "PP[RES+CONTENSOR]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1}"
    u = philox_np.uniforms(94, 96, 8)
    r = run_weights(CARD_RES_SCR, u, REPLAY_F + ["--nbt", "1024", "--nkt2", "10000"], proc=proc,
                    dim=6)
    save("rcf_screened_15x12_weights.npz", seed=94, u=u, card=os.path.basename(CARD_RES_SCR),
         proc=proc, n_bt=1024, n_kt2=10000, loop_kt=15, loop_phi=12, loop_ktmax=1.75, **r)


def nbody_fixtures():
    """Regge continuum of four central particles (PP[CON]<F> -> 4 bodies, MRegge::ME6 with
    NBodyPhaseSpace): pi+ pi- pi+ pi- and pi+ pi- K+ K- at tree level, the screened
    amplitude, and the reference's VEGAS cross section of the 4 pi process. The generator
    draws inside EventWeight, in order: four off-shell masses of the stable central
    particles (inert, 0.5), the two intermediate masses u[6], u[7], the acceptance draw of the
    weighted N-body setup (inert, 0.5), then (cos theta, phi) of three decays, u[8..13]."""
    replay = ["--replay", "h,h,h,h,6,7,h,8,9,10,11,12,13"]
    proc4 = "PP[CON]<F> -> pi+ pi- pi+ pi-"
    cases = [("f4_tree_weights.npz", 111, 2048, CARD, proc4),
             ("f4_kk_tree_weights.npz", 112, 1024, CARD, "PP[CON]<F> -> pi+ pi- K+ K-")]
    for name, seed, n, card, proc in cases:
        u = philox_np.uniforms(seed, n, 14)
        r = run_weights(card, u, replay, proc=proc, dim=6, leaves=4)
        save(name, seed=seed, u=u, card=os.path.basename(card), proc=proc, **r)
    u = philox_np.uniforms(113, 96, 14)
    r = run_weights(CARD_SCR, u, replay + ["--nbt", "1024", "--nkt2", "10000"], proc=proc4,
                    dim=6, leaves=4)
    save("f4_screened_weights.npz", seed=113, u=u, card=os.path.basename(CARD_SCR), proc=proc4,
         n_bt=1024, n_kt2=10000, **r)
    # Cross section of the 4 pi process. The integrand is heavy-tailed (in flat sampling the
    # top 100 of 4e5 points carry 90% of the integral), and the reference's VEGAS (6
    # dimensions, the 8 decay draws inside EventWeight) settles on 1.67e-10 b +- 0.1%, a
    # factor 8 below the mean of its own EventWeight over uniform points. The fixture keeps
    # both: the VEGAS number and the flat-sampling mean of the reference's EventWeight (its
    # own generator draws) over 8 x 5e5 Philox points, with its standard error.
    out = subprocess.run([REF_BIN, "vegas", CARD, proc4, "--cores", "8"], check=True,
                         capture_output=True, text=True).stdout
    line = [l for l in out.splitlines() if l.startswith("RESULT")][-1]
    vegas = list(map(float, line.split()[1:3]))
    os.makedirs(TMP, exist_ok=True)
    procs, parts = [], []
    for k in range(8):
        uf, wf = os.path.join(TMP, "f%d.bin" % k), os.path.join(TMP, "fw%d.bin" % k)
        philox_np.uniforms(120 + k, 500000, 6).astype(np.float64).tofile(uf)
        procs.append(subprocess.Popen([REF_BIN, "weights", CARD, proc4, uf, "6", wf],
                                      stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL))
        parts.append(wf)
    for pr in procs:
        assert pr.wait() == 0
    w = np.concatenate([np.fromfile(f).reshape(-1, 24)[:, 0] for f in parts])
    flat = [float(w.mean()), float(w.std() / np.sqrt(len(w)))]
    with open(os.path.join(HERE, "f4_sigma.json"), "w") as fh:
        json.dump({"process": proc4, "card": os.path.basename(CARD), "flat_points": len(w),
                   "flat_sigma_barn": flat[0], "flat_sigma_err_barn": flat[1],
                   "vegas_sigma_barn": vegas[0], "vegas_sigma_err_barn": vegas[1]}, fh, indent=1)
    print("f4: flat", flat, "vegas", vegas)


def nbody6_fixtures():
    """Regge continuum of six central particles (PP[CON] -> pi+ pi- pi+ pi- pi+ pi-,
    MRegge::ME8) in both classes, tree level and screened. Factorized class: the generator
    draws inside EventWeight, in order, are six inert off-shell masses (0.5), the four
    intermediate masses of NBodySetup u[6..9], its acceptance draw (inert, 0.5) and
    (cos theta, phi) of five decays u[10..19]; continuum class: the six inert masses."""
    proc_f = "PP[CON]<F> -> pi+ pi- pi+ pi- pi+ pi-"
    proc_c = "PP[CON]<C> -> pi+ pi- pi+ pi- pi+ pi-"
    rep_f = ["--replay", "h,h,h,h,h,h,6,7,8,9,h," + ",".join(str(k) for k in range(10, 20))]
    rep_c = ["--replay", "h,h,h,h,h,h"]
    scr = ["--nbt", "1024", "--nkt2", "10000"]
    u = philox_np.uniforms(161, 1024, 20)
    r = run_weights(CARD, u, rep_f, proc=proc_f, dim=6, leaves=6)
    save("f6_tree_weights.npz", seed=161, u=u, card=os.path.basename(CARD), proc=proc_f, **r)
    u = philox_np.uniforms(162, 1024, 20)
    r = run_weights(CARD, u, rep_c, proc=proc_c, leaves=6)
    save("c6_tree_weights.npz", seed=162, u=u, card=os.path.basename(CARD), proc=proc_c, **r)
    u = philox_np.uniforms(163, 384, 20)
    r = run_weights(CARD_SCR, u, rep_f + scr, proc=proc_f, dim=6, leaves=6)
    save("f6_screened_weights.npz", seed=163, u=u, card=os.path.basename(CARD_SCR), proc=proc_f,
         n_bt=1024, n_kt2=10000, **r)
    u = philox_np.uniforms(164, 64, 20)
    r = run_weights(CARD_SCR, u, rep_c + scr, proc=proc_c, leaves=6)
    save("c6_screened_weights.npz", seed=164, u=u, card=os.path.basename(CARD_SCR), proc=proc_c,
         n_bt=1024, n_kt2=10000, **r)


def veto_fixtures():
    """Veto cuts (VETOCUTS; MProcess::VetoCuts on the final-state leaves) with two domains, for
    the <C> pi+ pi- continuum, the tensor rho rho cascade (its four pions) and the 4 pi
    continuum (<F>)."""
    card = os.path.join(HERE, "cards", "pp_con_pipi_veto.json")
    cases = [("veto_c_weights.npz", 141, "PP[CON]<C> -> pi+ pi-", [], 8, 8),
             ("veto_rr_weights.npz", 142,
              "PP[CONTENSOR]<F> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}",
              ["--replay", "h,h,8,h,h,9,6,7,h,h,10,11,h,h,12,13"], 6, 14),
             ("veto_f4_weights.npz", 143, "PP[CON]<F> -> pi+ pi- pi+ pi-",
              ["--replay", "h,h,h,h,6,7,h,8,9,10,11,12,13"], 6, 14)]
    for name, seed, proc, extra, dim, width in cases:
        u = philox_np.uniforms(seed, 2048, width)
        r = run_weights(card, u, extra, proc=proc, dim=dim)
        save(name, seed=seed, u=u, card=os.path.basename(card), proc=proc, **r)


def nbody_c_fixtures():
    """Regge continuum of four central particles in the continuum class (PP[CON]<C> ->
    pi+ pi- pi+ pi-, MRegge::ME6 with MContinuum::BNRandomKin / BNBuildKin): tree level and
    screened. The generator draws inside EventWeight are the four inert off-shell masses."""
    replay = ["--replay", "h,h,h,h"]
    proc = "PP[CON]<C> -> pi+ pi- pi+ pi-"
    u = philox_np.uniforms(131, 2048, 14)
    r = run_weights(CARD, u, replay, proc=proc, leaves=4)
    save("c4_tree_weights.npz", seed=131, u=u, card=os.path.basename(CARD), proc=proc, **r)
    u = philox_np.uniforms(132, 64, 14)
    r = run_weights(CARD_SCR, u, replay + ["--nbt", "1024", "--nkt2", "10000"], proc=proc,
                    leaves=4)
    save("c4_screened_weights.npz", seed=132, u=u, card=os.path.basename(CARD_SCR), proc=proc,
         n_bt=1024, n_kt2=10000, **r)


def regge_res_fixtures():
    """Regge resonances (PROC_9 PP[RES], PROC_17 PP[RES+CON]; MRegge::ME3 with the spin
    density-matrix production and decay amplitudes): the Collins-Soper, helicity and
    non-rotated frames, a JZ density override, SPINGEN off, K+ K- (f0(980) below threshold),
    <C>, and the screened amplitude."""
    REPLAY_F = ["--replay", "h,h,6,7"]
    cases = [
        ("gr_tree_weights.npz", 101, 1024, CARD_RES,
         "PP[RES]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1}", REPLAY_F, 6),
        ("grc_tree_weights.npz", 102, 1024, CARD_RES,
         "PP[RES+CON]<F> -> pi+ pi- @RES{f0_500:1, f0_980:1, f2_1270:1, f2_1525:1}", REPLAY_F, 6),
        ("grc_hx_tree_weights.npz", 103, 512, CARD_RES,
         "PP[RES+CON]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1} @FRAME:HX", REPLAY_F, 6),
        ("grc_cm_jz_tree_weights.npz", 104, 512, CARD_RES,
         "PP[RES+CON]<F> -> pi+ pi- @RES{f2_1270:1} @FRAME:CM @R[f2_1270]{JZ0:1, JZ1:0.5, JZ2:0.2}",
         REPLAY_F, 6),
        ("grc_nogen_tree_weights.npz", 105, 512, CARD_RES,
         "PP[RES+CON]<F> -> pi+ pi- @RES{f2_1270:1, f2_1950:1} @SPINGEN:false", REPLAY_F, 6),
        ("grc_kk_tree_weights.npz", 106, 512, CARD_RES,
         "PP[RES+CON]<F> -> K+ K- @RES{f0_980:1, f2_1270:1, f2_1525:1}", REPLAY_F, 6),
        ("grc_c_tree_weights.npz", 107, 1024, CARD_RES,
         "PP[RES+CON]<C> -> pi+ pi- @RES{f0_980:1, f2_1270:1}", [], 8),
    ]
    for name, seed, n, card, proc, extra, dim in cases:
        u = philox_np.uniforms(seed, n, 8)
        r = run_weights(card, u, extra, proc=proc, dim=dim)
        save(name, seed=seed, u=u, card=os.path.basename(card), proc=proc, **r)
    proc = "PP[RES+CON]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1}"
    u = philox_np.uniforms(108, 96, 8)
    r = run_weights(CARD_RES_SCR, u, REPLAY_F + ["--nbt", "1024", "--nkt2", "10000"], proc=proc,
                    dim=6)
    save("grc_screened_15x12_weights.npz", seed=108, u=u, card=os.path.basename(CARD_RES_SCR),
         proc=proc, n_bt=1024, n_kt2=10000, loop_kt=15, loop_phi=12, loop_ktmax=1.75, **r)
    # VEGAS cross section (reference ranlux48 points, 8 threads)
    proc = "PP[RES+CON]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1}"
    out = subprocess.run([REF_BIN, "vegas", CARD_RES, proc, "--cores", "8"], check=True,
                         capture_output=True, text=True).stdout
    write_sigma("grc_vegas_sigma.json", out, proc, os.path.basename(CARD_RES))


def write_sigma(name, out, proc, card):
    line = [l for l in out.splitlines() if l.startswith("RESULT")][-1]
    sigma, err = map(float, line.split()[1:3])
    with open(os.path.join(HERE, name), "w") as f:
        json.dump({"process": proc, "card": card, "sigma_barn": sigma, "sigma_err_barn": err,
                   "ncall": 100000, "iter": 5, "precision": 0.001}, f, indent=1)
    print(name, "sigma", sigma, "+-", err)


def cascade_fixtures():
    """Vector-meson pairs with two-body cascades (<F>, 14 dimensions): tensor-pomeron 2xV
    (MTensorPomeron::ME4) and Regge continuum rho rho -> pi+ pi- pi+ pi-, tensor phi phi ->
    K+ K- K+ K-, and the screened tensor rho rho. Replay order of the reference's draws: the
    two daughter masses then the mass of each central particle (u[8], u[9]), the central
    decay angles (u[6], u[7]), then per central particle its daughters' masses and decay
    angles (u[10..11], u[12..13]); daughter masses of width ~1e-17 GeV take 0.5."""
    REPLAY = ["--replay", "h,h,8,h,h,9,6,7,h,h,10,11,h,h,12,13"]
    RR = "rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}"
    cases = [
        ("rr_tree_weights.npz", 81, 2048, CARD, "PP[CONTENSOR]<F> -> " + RR),
        ("rr_regge_tree_weights.npz", 82, 1024, CARD, "PP[CON]<F> -> " + RR),
        ("ff_tree_weights.npz", 83, 512, CARD,
         "PP[CONTENSOR]<F> -> phi(1020)0 > {K+ K-} phi(1020)0 > {K+ K-}"),
    ]
    for name, seed, n, card, proc in cases:
        u = philox_np.uniforms(seed, n, 14)
        r = run_weights(card, u, REPLAY, proc=proc, dim=6, leaves=4)
        save(name, seed=seed, u=u, card=os.path.basename(card), proc=proc, **r)
    proc = "PP[CONTENSOR]<F> -> " + RR
    u = philox_np.uniforms(84, 256, 14)
    r = run_weights(CARD_SCR, u, REPLAY + ["--nbt", "1024", "--nkt2", "10000"], proc=proc, dim=6,
                    leaves=4)
    save("rr_screened_15x12_weights.npz", seed=84, u=u, card=os.path.basename(CARD_SCR),
         proc=proc, n_bt=1024, n_kt2=10000, loop_kt=15, loop_phi=12, loop_ktmax=1.75, **r)
    # VEGAS cross section of the tensor rho rho process (reference ranlux48 points, 8 threads)
    out = subprocess.run([REF_BIN, "vegas", CARD, proc, "--cores", "8"], check=True,
                         capture_output=True, text=True).stdout
    write_sigma("rr_vegas_sigma.json", out, proc, os.path.basename(CARD))


def ccascade_fixtures():
    """Vector-meson pair cascades in the continuum class <C> (BNRandomKin draws the off-shell
    masses, BNBuildKin decays the central pair with ConstructDecayKinematics), and <F> with
    @OFFSHELL:0. Replay order of the reference's draws in <C>: per central particle its two
    daughters' masses, then its own mass (GetOffShellMass, u[8] and u[9] unless OFFSHELL = 0,
    where the Breit-Wigner collapses to the pole mass and the value is 0.5); then per central
    particle its daughters' masses and its decay angles (the four coordinates after the 8 of
    the 2-body point, or after the two masses). Pion masses (width ~1e-17 GeV) take 0.5."""
    RR = "rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}"
    REPLAY_C12 = ["--replay", "h,h,h,h,h,h,h,h,8,9,h,h,10,11"]
    REPLAY_C14 = ["--replay", "h,h,8,h,h,9,h,h,10,11,h,h,12,13"]
    REPLAY_F12 = ["--replay", "h,h,h,h,h,h,6,7,h,h,8,9,h,h,10,11"]
    cases = [
        ("rrc_tree_weights.npz", 91, 2048, CARD, "PP[CONTENSOR]<C> -> " + RR + " @OFFSHELL:0",
         12, 8, REPLAY_C12),
        ("rrc_regge_tree_weights.npz", 92, 1024, CARD, "PP[CON]<C> -> " + RR + " @OFFSHELL:0",
         12, 8, REPLAY_C12),
        ("rrc14_tree_weights.npz", 93, 1024, CARD, "PP[CONTENSOR]<C> -> " + RR, 14, 8,
         REPLAY_C14),
        ("rrf12_tree_weights.npz", 94, 1024, CARD, "PP[CONTENSOR]<F> -> " + RR + " @OFFSHELL:0",
         12, 6, REPLAY_F12),
    ]
    for name, seed, n, card, proc, D, pdim, rep in cases:
        u = philox_np.uniforms(seed, n, D)
        r = run_weights(card, u, rep, proc=proc, dim=pdim, leaves=4)
        save(name, seed=seed, u=u, card=os.path.basename(card), proc=proc, **r)
    proc = "PP[CONTENSOR]<C> -> " + RR + " @OFFSHELL:0"
    u = philox_np.uniforms(95, 256, 12)
    r = run_weights(CARD_SCR, u, REPLAY_C12 + ["--nbt", "1024", "--nkt2", "10000"], proc=proc,
                    dim=8, leaves=4)
    save("rrc_screened_15x12_weights.npz", seed=95, u=u, card=os.path.basename(CARD_SCR),
         proc=proc, n_bt=1024, n_kt2=10000, loop_kt=15, loop_phi=12, loop_ktmax=1.75, **r)
    out = subprocess.run([REF_BIN, "vegas", CARD, proc, "--cores", "8"], check=True,
                         capture_output=True, text=True).stdout
    write_sigma("rrc_vegas_sigma.json", out, proc, os.path.basename(CARD))


def excitation_fixtures():
    """Forward excitation (NSTARS = 1, 2; MProcess::SampleForwardMasses, PomPomProtonVertex,
    ForwardVolume) of the Regge pi+ pi- continuum, both classes, M^2 / s <= 0.05, 10-dimensional
    points: <C> u[8] (u[9]) the excited masses, single excitation's side draw u[9]; <F> u[6]
    (u[7]) the masses or the side draw, the decay angles u[8], u[9]. The specs below serve the
    draws the reference takes inside EventWeight, in order (two inert pion mass draws, the side,
    the decay angles); each was checked to be consumed exactly."""
    c1 = os.path.join(HERE, "cards", "pp_con_pipi_nstar1.json")
    c2 = os.path.join(HERE, "cards", "pp_con_pipi_nstar2.json")
    cs = os.path.join(HERE, "cards", "pp_con_pipi_nstar1_screened.json")
    PC, PF = "PP[CON]<C> -> pi+ pi-", "PP[CON]<F> -> pi+ pi-"
    cases = [("nstar1_c_tree_weights.npz", 221, c1, PC, "h,h,9", 9),
             ("nstar2_c_tree_weights.npz", 222, c2, PC, "h,h", 10),
             ("nstar1_f_tree_weights.npz", 223, c1, PF, "h,h,7,8,9", 7),
             ("nstar2_f_tree_weights.npz", 224, c2, PF, "h,h,8,9", 8)]
    for name, seed, card, proc, spec, dim in cases:
        u = philox_np.uniforms(seed, 1024, 10)
        r = run_weights(card, u, ["--replay", spec], proc=proc, dim=dim)
        save(name, seed=seed, u=u, card=os.path.basename(card), proc=proc, **r)
    u = philox_np.uniforms(225, 128, 10)
    r = run_weights(cs, u, ["--replay", "h,h,9", "--nbt", "1024", "--nkt2", "10000"], proc=PC,
                    dim=9)
    save("nstar1_c_screened_15x12_weights.npz", seed=225, u=u, card=os.path.basename(cs),
         proc=PC, n_bt=1024, n_kt2=10000, loop_kt=15, loop_phi=12, loop_ktmax=1.75, **r)


def ld_fixtures():
    """The oracle restatement in long double arithmetic (oracle/_build/liborc_ld.so: the same
    formulas and constants as the reference, 64-bit significands on x86) on the points of every
    weight fixture: long_double_oracle.npz holds, per fixture, the weights nearer the exact value of the
    reference's formulas than any FP64 evaluation (the reference's own or the engine's)."""
    sys.path.insert(0, REPO)
    sys.path.insert(0, HERE)
    from oracle import oracle_api as orc
    from fixture_meta import fixture_params, weight_fixtures
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle")])
    out = {}
    for f in weight_fixtures():
        g = np.load(os.path.join(HERE, f))
        P, msa = fixture_params(f, g)
        w, _ = orc.weights(P, g["u"], msa=msa, nthreads=8, long_double=True)
        out[f[:-len(".npz")]] = w
        nz = g["w"] > 0
        print("%-34s reference vs long double: max rel %.2e" %
              (f, np.max(np.abs(g["w"][nz] - w[nz]) / w[nz]) if nz.any() else 0.0))
    np.savez_compressed(os.path.join(HERE, "long_double_oracle.npz"), **out)
    print("wrote long_double_oracle.npz")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=REF_DEFAULT)
    ap.add_argument("--only", choices=["all", "resonances", "cascades", "rescon", "regge_res",
                                       "nbody", "nbody_c", "nbody6", "veto", "ccascades",
                                       "ld", "excitation"],
                    default="all")
    a = ap.parse_args()
    if a.only == "ld":  # needs only the oracle
        ld_fixtures()
        return
    subprocess.check_call(["make", "-s", "-C", os.path.join(REPO, "oracle", "refbuild"), "-j8",
                           "REF=" + a.ref])
    if a.only in ("all", "nbody6"):
        nbody6_fixtures()
    if a.only == "nbody6":
        return
    if a.only in ("all", "excitation"):
        excitation_fixtures()
    if a.only == "excitation":
        ld_fixtures()
        return
    if a.only == "all":
        ld_fixtures()
    if a.only in ("all", "ccascades"):
        ccascade_fixtures()
    if a.only == "ccascades":
        return
    if a.only in ("all", "veto"):
        veto_fixtures()
    if a.only == "veto":
        return
    if a.only in ("all", "nbody_c"):
        nbody_c_fixtures()
    if a.only == "nbody_c":
        return
    if a.only in ("all", "nbody"):
        nbody_fixtures()
    if a.only == "nbody":
        return
    if a.only in ("all", "regge_res"):
        regge_res_fixtures()
    if a.only == "regge_res":
        return
    if a.only in ("all", "rescon"):
        rescon_fixtures()
    if a.only == "rescon":
        return
    if a.only in ("all", "cascades"):
        cascade_fixtures()
    if a.only == "cascades":
        return
    resonance_fixtures()
    if a.only == "resonances":
        return

    # c1: tree-level weights, TUNE0 (power-law off-shell form factor) and the
    # exponential form-factor variant.
    u = philox_np.uniforms(1, 4096, 8)
    r = run_weights(CARD, u)
    save("c1_tune0_weights.npz", seed=1, u=u, **r)
    u = philox_np.uniforms(2, 1024, 8)
    r = run_weights(CARD, u, ["--offshellff", "0"])
    save("c1_expff_weights.npz", seed=2, u=u, **r)
    u = philox_np.uniforms(3, 512, 8)
    r = run_weights(CARD, u, ["--offshellff", "1"])
    save("c1_orearff_weights.npz", seed=3, u=u, **r)

    # Edge points: hypercube corners and faces (u = 0 exactly and u -> 1).
    edge = []
    for v in (0.0, 1.0 - 2.0**-53, 0.5):
        edge.append(np.full(8, v))
    rng = np.random.default_rng(5)
    for _ in range(61):
        x = rng.random(8)
        k = rng.integers(0, 8, size=2)
        x[k[0]] = 0.0
        x[k[1]] = 1.0 - 2.0**-53
        edge.append(x)
    u = np.array(edge)
    r = run_weights(CARD, u)
    save("c1_edge_weights.npz", u=u, **r)

    # Eikonal tables: 1024 impact-parameter intervals, 10000 kt^2 intervals.
    os.makedirs(TMP, exist_ok=True)
    tf = os.path.join(TMP, "eik.bin")
    subprocess.run([REF_BIN, "eikonal", CARD_SCR, PROC, tf, "--nbt", "1024", "--nkt2", "10000"],
                   check=True, capture_output=True)
    e = np.fromfile(tf)
    xs = e[:3]
    mbt = e[3:3 + 1025 * 3].reshape(-1, 3)
    msa = e[3 + 1025 * 3:].reshape(-1, 3)
    save("eikonal_nbt1024_nkt10000.npz", xs=xs, mbt=mbt, msa=msa)
    # Default numerics (10000 x 10000): cross sections only.
    subprocess.run([REF_BIN, "eikonal", CARD_SCR, PROC, tf], check=True, capture_output=True)
    e = np.fromfile(tf)
    save("eikonal_default_xs.npz", xs=e[:3], mbt_rows=np.array(10001), msa_rows=np.array(10001))

    # c2: screened weights. Loop grid 63 kt x 33 phi intervals (64 x 34 points),
    # kt <= 3 GeV; and the reference default grid (15 x 12, kt <= 1.75 GeV).
    u = philox_np.uniforms(11, 96, 8)
    r = run_weights(CARD_SCR, u, ["--nbt", "1024", "--nkt2", "10000", "--loopkt", "63",
                                  "--loopphi", "33", "--maxloopkt", "3.0"])
    save("c2_screened_63x33_weights.npz", seed=11, u=u, n_bt=1024, n_kt2=10000, loop_kt=63,
         loop_phi=33, loop_ktmax=3.0, **r)
    u = philox_np.uniforms(12, 96, 8)
    r = run_weights(CARD_SCR, u, ["--nbt", "1024", "--nkt2", "10000"])
    save("c2_screened_15x12_weights.npz", seed=12, u=u, n_bt=1024, n_kt2=10000, loop_kt=15,
         loop_phi=12, loop_ktmax=1.75, **r)

    # <F>: factorized phase space, decay angles lifted into u[6], u[7].
    PROC_F = "PP[CON]<F> -> pi+ pi-"
    REPLAY_F = ["--replay", "h,h,6,7"]
    u = philox_np.uniforms(31, 2048, 8)
    r = run_weights(CARD, u, REPLAY_F, proc=PROC_F, dim=6)
    save("f_tree_weights.npz", seed=31, u=u, **r)
    u = philox_np.uniforms(32, 96, 8)
    r = run_weights(CARD_SCR, u, REPLAY_F + ["--nbt", "1024", "--nkt2", "10000"], proc=PROC_F,
                    dim=6)
    save("f_screened_15x12_weights.npz", seed=32, u=u, n_bt=1024, n_kt2=10000, loop_kt=15,
         loop_phi=12, loop_ktmax=1.75, **r)

    # Tensor-pomeron continuum of pi+ pi- (PROC_12, MTensorPomeron::ME4 2xS), <C> and <F>.
    PROC_T = "PP[CONTENSOR]<C> -> pi+ pi-"
    u = philox_np.uniforms(41, 2048, 8)
    r = run_weights(CARD, u, proc=PROC_T)
    save("t_tree_weights.npz", seed=41, u=u, **r)
    u = philox_np.uniforms(42, 1024, 8)
    r = run_weights(CARD, u, REPLAY_F, proc="PP[CONTENSOR]<F> -> pi+ pi-", dim=6)
    save("tf_tree_weights.npz", seed=42, u=u, **r)
    u = philox_np.uniforms(43, 96, 8)
    r = run_weights(CARD_SCR, u, ["--nbt", "1024", "--nkt2", "10000"], proc=PROC_T)
    save("t_screened_15x12_weights.npz", seed=43, u=u, n_bt=1024, n_kt2=10000, loop_kt=15,
         loop_phi=12, loop_ktmax=1.75, **r)

    # VEGAS integration of c1 (reference ranlux48 points, 8 threads).
    out = subprocess.run([REF_BIN, "vegas", CARD, PROC, "--cores", "8"], check=True,
                         capture_output=True, text=True).stdout
    line = [l for l in out.splitlines() if l.startswith("RESULT")][-1]
    sigma, err = map(float, line.split()[1:3])
    with open(os.path.join(HERE, "c1_vegas_sigma.json"), "w") as f:
        json.dump({"process": PROC, "card": "cards/pp_con_pipi.json", "sigma_barn": sigma,
                   "sigma_err_barn": err, "ncall": 100000, "iter": 5, "precision": 0.001}, f,
                  indent=1)
    print("c1 VEGAS sigma", sigma, "+-", err)


if __name__ == "__main__":
    main()

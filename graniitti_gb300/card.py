"""Steering-card reader: the generator's JSON5 cards -> engine parameters.

Mirrors what MGraniitti::ReadInput and MProcess::post_Constructor derive from a
card (src/MGraniitti.cc:318-963, src/MContinuum.cc:64-89), for the process family
the engine implements. The card layout (GENERALPARAM, PROCESSPARAM,
INTEGRALPARAM, GENCUTS, FIDCUTS, VETOCUTS blocks) is the generator's own so that
existing cards run unchanged.
"""
import json
import math
import re

import numpy as np

from . import _abi
from .modeldata import BRANCHING, PARTICLES, RESONANCES, SPIN, TUNES, VECTOR_COUPLING

_PROC_RE = re.compile(r"^\s*([A-Za-z]+)\[([A-Z+]+)\]<([A-Z])>\s*$")


def strip_json5(text):
    """Remove // and /* */ comments and trailing commas (MAux.cc:309-340)."""
    out = []
    i, n = 0, len(text)
    in_str = False
    while i < n:
        ch = text[i]
        if in_str:
            out.append(ch)
            if ch == "\\" and i + 1 < n:
                out.append(text[i + 1])
                i += 2
                continue
            if ch == '"':
                in_str = False
            i += 1
            continue
        if ch == '"':
            in_str = True
            out.append(ch)
            i += 1
        elif text.startswith("//", i):
            j = text.find("\n", i)
            i = n if j < 0 else j
        elif text.startswith("/*", i):
            j = text.find("*/", i + 2)
            i = n if j < 0 else j + 2
        else:
            out.append(ch)
            i += 1
    s = "".join(out)
    return re.sub(r",(\s*[}\]])", r"\1", s)


def read_card(path):
    with open(path) as f:
        return json.loads(strip_json5(f.read()))


def split_commands(proc):
    """The '@' commands of a process string (aux::SplitCommands, src/MAux.cc:690-800):
    '@ID[t1,t2]{k1:v1, k2:v2}' -> (ID, [t1, t2], {k1: v1, k2: v2}); a singlet '@ID:VALUE'
    (or '@ID') -> (ID, [], {'_SINGLET_': VALUE or 'true'})."""
    if "@" not in proc:
        return []
    out = []
    for blk in proc[proc.index("@"):].split("@")[1:]:
        blk = " ".join(blk.split())
        targets, args = [], {}
        if ("[" in blk) != ("]" in blk):
            raise ValueError("incomplete @ID[]{} syntax: %r" % blk)
        if "[" in blk:
            l, r = blk.index("["), blk.index("]")
            targets = [t.strip() for t in blk[l + 1:r].split(",") if t.strip()]
            blk = blk[:l] + blk[r + 1:]
        if ("{" in blk) != ("}" in blk):
            raise ValueError("incomplete @ID[]{} syntax: %r" % blk)
        if "{" in blk:
            l, r = blk.index("{"), blk.index("}")
            ident = blk[:l].strip()
            for kv in blk[l + 1:r].split(","):
                if kv.strip():
                    if ":" not in kv:
                        raise ValueError("@%s{} argument %r is not key:value" % (ident, kv))
                    k, v = kv.split(":", 1)
                    args[k.strip()] = v.strip()
        else:
            parts = blk.split(":")
            ident = parts[0].strip()
            if len(parts) > 2:
                raise ValueError("invalid @ singlet %r" % blk)
            args["_SINGLET_"] = parts[1].strip() if len(parts) == 2 else "true"
        out.append((ident, targets, args))
    return out


def parse_process(proc):
    """'PP[CON]<C> -> pi+ pi-' -> (istate, channel, class, [final states], options);
    options holds the singlet '@ID:VALUE' commands (split_commands gives all of them)."""
    opts = {}
    if "@" in proc:
        for ident, _, args in split_commands(proc):
            if "_SINGLET_" in args:
                opts[ident] = args["_SINGLET_"]
        proc = proc[:proc.index("@")]
    if "->" not in proc:
        raise ValueError("process string needs '->': %r" % proc)
    left, right = proc.split("->", 1)
    m = _PROC_RE.match(left)
    if not m:
        raise ValueError("cannot parse process %r" % left)
    finals = [name for name, _ in decay_tree(right)]
    return m.group(1), m.group(2), m.group(3), finals, opts


def decay_tree(text):
    """'rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}' -> [(name, [daughters]), ...], the
    decay syntax of the process string (MProcess::SetDecayMode, src/MProcess.cc:355-440)."""
    toks = text.replace("{", " { ").replace("}", " } ").split()

    def items(i, closing):
        out = []
        while i < len(toks):
            t = toks[i]
            if t == "}":
                if not closing:
                    raise ValueError("unbalanced '}' in %r" % text)
                return out, i + 1
            if t in (">", "{"):
                raise ValueError("decay syntax error at %r in %r" % (t, text))
            name, i = t, i + 1
            kids = []
            if i < len(toks) and toks[i] == ">":
                if i + 1 >= len(toks) or toks[i + 1] != "{":
                    raise ValueError("'>' must be followed by '{...}' in %r" % text)
                kids, i = items(i + 2, True)
            out.append((name, kids))
        if closing:
            raise ValueError("unbalanced '{' in %r" % text)
        return out, i

    return items(0, False)[0]


class UnsupportedProcess(ValueError):
    pass


def build_params(card, process=None, tune=None):
    """Engine ProcessParams from a parsed card (dict) and an optional process override."""
    P = _abi.ProcessParams()
    gp = card["GENERALPARAM"]
    pp = card["PROCESSPARAM"]
    tune = tune or gp.get("MODELPARAM", "TUNE0")
    if tune not in TUNES:
        raise UnsupportedProcess("model tune %s is not bundled" % tune)
    T = TUNES[tune]
    proc = process or pp["PROCESS"]
    istate, channel, cls, finals, _ = parse_process(proc)
    tree = decay_tree(proc.split("@")[0].split("->", 1)[1])
    casc = [kids for _, kids in tree]
    if any(casc):
        # two-body cascades "a > {c d} b > {e f}" of both central particles (<C> and <F>)
        if not (all(len(k) == 2 and all(not g for _, g in k) for k in casc) and len(casc) == 2):
            raise UnsupportedProcess("decay trees: both central particles decay to two stable "
                                     "particles")
        if channel == "RESTENSOR":
            raise UnsupportedProcess("RESTENSOR decays directly to two pseudoscalars")
    elif any(f in PARTICLES and PARTICLES[f][2] > 1e-6 for f in finals):
        # the reference draws Breit-Wigner masses for them (MProcess::GetOffShellMass)
        raise UnsupportedProcess("unstable central particles need their decays: a > {c d}")
    nbody = len(finals) in (4, 6) and channel == "CON" and not any(casc)
    if not (istate == "PP" and channel in ("CON", "RES", "RES+CON", "CONTENSOR", "RESTENSOR",
                                           "RES+CONTENSOR") and
            cls in ("C", "F") and (len(finals) == 2 or nbody)):
        raise UnsupportedProcess(
            "engine implements PP[CON|RES|RES+CON|CONTENSOR|RESTENSOR|RES+CONTENSOR]<C|F> -> "
            "2-body and PP[CON]<C|F> -> 4- and 6-body, got %r" % proc)
    if nbody and any(SPIN.get(f, 0) != 0 for f in finals):
        raise UnsupportedProcess("4- and 6-body central states of spin-0 particles")
    vec = all(SPIN.get(f, 0) == 1 for f in finals)
    if channel == "CONTENSOR" and not (
            all(f in ("pi+", "pi-", "K+", "K-", "pi0") for f in finals) or
            (vec and finals[0] == finals[1] and finals[0] in VECTOR_COUPLING)):
        raise UnsupportedProcess("CONTENSOR is implemented for pseudoscalar pairs (2xS) and "
                                 "rho rho / phi phi (2xV)")
    if channel in ("RES", "RES+CON", "RESTENSOR", "RES+CONTENSOR") and \
            sorted(finals) not in (["pi+", "pi-"], ["K+", "K-"]):
        raise UnsupportedProcess("%s is implemented for pi+ pi- and K+ K- decays" % channel)
    nstars = int(pp.get("NSTARS", 0))
    if nstars not in (0, 1, 2):
        raise ValueError("NSTARS must be 0, 1 or 2")
    if nstars and not (channel == "CON" and len(finals) == 2 and not any(casc)):
        raise UnsupportedProcess("forward excitation (NSTARS > 0) is implemented for the Regge "
                                 "continuum of two central particles")
    if pp["BEAM"] != ["p+", "p+"]:
        raise UnsupportedProcess("beams other than p+ p+ are not implemented")
    E1, E2 = float(pp["ENERGY"][0]), float(pp["ENERGY"][1])
    if E1 != E2:
        raise UnsupportedProcess("asymmetric beams are not implemented")
    mb = PARTICLES["p+"][1]
    E1 = max(E1, 1.001 * mb)
    # s = (pbeam1 + pbeam2)^2 with equal energies (MProcess.cc:309-324)
    P.sqrt_s = 2.0 * E1
    P.m_beam = mb
    P.process = {"CON": _abi.GRN_PROC_REGGE_CON, "CONTENSOR": _abi.GRN_PROC_TENSOR_CON,
                 "RESTENSOR": _abi.GRN_PROC_TENSOR_RES,
                 "RES+CONTENSOR": _abi.GRN_PROC_TENSOR_RESCON,
                 "RES": _abi.GRN_PROC_REGGE_RES, "RES+CON": _abi.GRN_PROC_REGGE_RESCON}[channel]
    P.phase_space = _abi.GRN_PS_CONTINUUM if cls == "C" else _abi.GRN_PS_FACTORIZED
    P.n_central = len(finals)
    P.screening = 1 if pp.get("POMLOOP", False) else 0
    for k, name in enumerate(finals):
        if name not in PARTICLES:
            raise UnsupportedProcess("unknown final state %s" % name)
        P.m_central[k] = PARTICLES[name][1]
    # identical-particle factor: product of the multiplicities' factorials (MProcess.cc:449-468)
    P.s_factor = float(np.prod([math.factorial(finals.count(f)) for f in sorted(set(finals))]))
    P.central_spin = 1 if vec else 0
    # @OFFSHELL:x, widths of the cascades' Breit-Wigner mass draws (MProcess::SetOFFSHELL,
    # src/MGraniitti.cc:588); the reference default (5) otherwise
    for ident, _, args in split_commands(proc):
        if ident == "OFFSHELL":
            P.offshell_user = 1
            P.offshell = float(args["_SINGLET_"])
    if any(casc):
        P.n_decay = 2
        for k, name in enumerate(finals):
            P.width[k] = PARTICLES[name][2]
        for k, (name, _) in enumerate(casc[0] + casc[1]):
            if name not in PARTICLES:
                raise UnsupportedProcess("unknown final state %s" % name)
            P.m_daughter[k] = PARTICLES[name][1]

    # Generation cuts with post_Constructor defaults (MContinuum.cc:64-89,
    # MProcess.cc:1369-1386).
    g = card.get("GENCUTS", {}).get("<C>", {})
    rap = g.get("Rap", [-9.0, 9.0])
    P.gcuts.rap_min, P.gcuts.rap_max = rap
    kt = g.get("Kt", [0.0, 10.0 / len(finals)])
    P.gcuts.kt_min, P.gcuts.kt_max = kt
    # forward pT: the technical boundary of MProcess::SetTechnicalBoundaries (src/MProcess.cc:
    # 1369-1386) grows with the excitation (2.5, 50, 100 GeV) unless set by the user
    pt = g.get("Pt", [0.0, (2.5, 50.0, 100.0)[nstars]])
    P.gcuts.fpt_min, P.gcuts.fpt_max = pt
    # forward excitation (NSTARS; GENCUTS "Xi" of the class: M^2 / s of an excited leg)
    P.excitation = nstars
    P.xi_max = 1.0
    xi = card.get("GENCUTS", {}).get("<%s>" % cls, {}).get("Xi")
    if xi is not None:
        if not (0.0 <= xi[0] <= xi[1] <= 1.0):
            raise ValueError("GENCUTS Xi must satisfy 0 <= min <= max <= 1")
        P.xi_max = float(xi[1])
    # <F>: system rapidity and mass windows (MGraniitti::ReadGenCuts; GENCUT defaults)
    gf = card.get("GENCUTS", {}).get("<F>", {})
    P.gcuts.Y_min, P.gcuts.Y_max = gf.get("Rap", [-9.0, 9.0])
    P.gcuts.M_min, P.gcuts.M_max = gf.get("M", [0.0, 0.0])
    if cls == "F":
        if "Rap" not in gf or "M" not in gf:
            raise ValueError('<F> needs "GENCUTS" : { "<F>" : { "Rap" : [..], "M" : [..] } }')
        P.gcuts.fpt_min, P.gcuts.fpt_max = gf.get("Pt", [0.0, (2.5, 50.0, 100.0)[nstars]])

    # Fiducial cuts (FIDCUT defaults, MKinematics.h:1579-1611).
    f = card.get("FIDCUTS", {})
    fc = P.fcuts
    fc.active = 1 if f.get("active", False) else 0
    defaults = dict(eta=(-30.0, 30.0), rap=(-30.0, 30.0), pt=(0.0, 1e6), Et=(0.0, 1e6),
                    M=(0.0, 1e6), Y=(-30.0, 30.0), Pt=(0.0, 1e6), ft=(0.0, 1e6), fM=(0.0, 1e6))
    part = f.get("PARTICLE", {})
    sysb = f.get("SYSTEM", {})
    fwd = f.get("FORWARD", {})
    vals = dict(defaults)
    if "Eta" in part: vals["eta"] = part["Eta"]
    if "Rap" in part: vals["rap"] = part["Rap"]
    if "Pt" in part: vals["pt"] = part["Pt"]
    if "Et" in part: vals["Et"] = part["Et"]
    if "M" in sysb: vals["M"] = sysb["M"]
    if "Rap" in sysb: vals["Y"] = sysb["Rap"]
    if "Pt" in sysb: vals["Pt"] = sysb["Pt"]
    if "t" in fwd: vals["ft"] = fwd["t"]
    if "M" in fwd: vals["fM"] = fwd["M"]
    for key, (lo, hi) in vals.items():
        setattr(fc, key + "_min", float(lo))
        setattr(fc, key + "_max", float(hi))
    # Veto domains "0", "1", ... with Eta and Pt ranges (MGraniitti::ReadVetoCuts,
    # src/MGraniitti.cc:921-962: the search stops at the first missing number)
    vc = card.get("VETOCUTS", {})
    P.veto_active = 1 if vc.get("active", False) else 0
    P.n_veto = 0
    if P.veto_active:
        doms = []
        while str(len(doms)) in vc and "Eta" in vc[str(len(doms))] and "Pt" in vc[str(len(doms))]:
            doms.append(vc[str(len(doms))])
        if len(doms) > _abi.GRN_MAX_VETO:
            raise UnsupportedProcess("at most %d veto domains" % _abi.GRN_MAX_VETO)
        for k, d in enumerate(doms):
            (P.veto_eta_min[k], P.veto_eta_max[k]), (P.veto_pt_min[k], P.veto_pt_max[k]) = \
                map(float, d["Eta"]), map(float, d["Pt"])
        P.n_veto = len(doms)

    # Model parameters.
    s = T["PARAM_SOFT"]
    P.soft.delta_P = s["DELTA_P"]
    P.soft.alpha_P = s["ALPHA_P"]
    P.soft.gN_P = s["gN_P"]
    P.soft.gN_O = s["gN_O"]
    P.soft.g3P = s["g3P"] * s["gN_P"]  # stored in the reference's convention (MForm.cc:132)
    P.soft.gamma = s["gamma"]
    P.soft.fc1, P.soft.fc2, P.soft.fc3 = s["fc1"], s["fc2"], s["fc3"]
    P.soft.odderon_on = 1 if s["ODDERON_ON"] else 0
    r = T["PARAM_REGGE"]
    for k in range(3):
        P.regge.a0[k] = r["a0"][k]
        P.regge.ap[k] = r["ap"][k]
        P.regge.sgn[k] = r["sgn"][k]
    P.regge.s0 = r["s0"]
    P.regge.offshellFF = r["offshellFF"]
    P.regge.b_EXP, P.regge.a_OREAR, P.regge.b_OREAR, P.regge.b_POW = (
        r["b_EXP"], r["a_OREAR"], r["b_OREAR"], r["b_POW"])
    cpl = T["COUPLINGS"][PARTICLES[finals[0]][3]]
    for k in range(3):
        P.regge.c[k] = cpl["c"][k]
        P.regge.active[k] = 1 if cpl["n"][k] else 0

    # Tensor-pomeron parameters (MTensorPomeronParam; pion or kaon coupling chosen by
    # the first central mass, MTensorPomeron.cc:730).
    tp = T["PARAM_TENSORPOM"]
    P.tensor.delta_P, P.tensor.ap_P, P.tensor.gPNN = tp["delta_P"], tp["ap_P"], tp["gPNN"]
    P.tensor.gPps = tp["gPpipi"] if P.m_central[0] < 0.2 else tp["gPKK"]
    P.tensor.em_kelly = 1 if T["PARAM_STRUCTURE"]["EM"] == "KELLY" else 0
    if vec and finals[0] in VECTOR_COUPLING:
        # pomeron-vector-vector couplings of rho or phi (MTensorPomeron.cc:811-823)
        P.tensor.gPvv[0], P.tensor.gPvv[1] = tp[VECTOR_COUPLING[finals[0]]]

    if channel in ("RESTENSOR", "RES+CONTENSOR"):
        set_resonances(P, pp, proc, tune, finals, allow_none=channel == "RES+CONTENSOR")
    if channel in ("RES", "RES+CON"):
        set_resonances(P, pp, proc, tune, finals, allow_none=channel == "RES+CON", regge=True)
    # spin correlations and frame of the Regge resonances (GENERAL.json PARAM_SPIN, then the
    # @SPINGEN / @SPINDEC / @FRAME commands, src/MGraniitti.cc:590-593)
    sp = dict(T.get("PARAM_SPIN", {"SPINGEN": True, "SPINDEC": True, "FRAME": "CS"}))
    for ident, _, args in split_commands(proc):
        if ident in ("SPINGEN", "SPINDEC"):
            sp[ident] = args.get("_SINGLET_", "true") == "true"
        elif ident == "FRAME":
            sp["FRAME"] = args.get("_SINGLET_", "")
    frames = {"CM": _abi.GRN_FRAME_CM, "HX": _abi.GRN_FRAME_HX, "CS": _abi.GRN_FRAME_CS}
    if sp["FRAME"] not in frames:
        raise UnsupportedProcess("spin frame %r (CM, HX and CS are implemented)" % sp["FRAME"])
    P.spin_gen, P.spin_dec = int(bool(sp["SPINGEN"])), int(bool(sp["SPINDEC"]))
    P.spin_frame = frames[sp["FRAME"]]
    P.omega = float(r.get("omega", 0.5))

    # Loop numerics: defaults 15 x 12 moved by 3*ND (MEikonal.h:40-57), tables
    # 10000 intervals (modeldata/NUMERICS.json).
    nd = int(card.get("INTEGRALPARAM", {}).get("POMLOOP", {}).get("ND", 0))
    P.loop.n_kt = max(3, 3 * nd + 15)
    P.loop.n_phi = max(3, 3 * nd + 12)
    P.loop.kt_min = 1e-4
    P.loop.kt_max = 1.75
    P.loop.n_bt = 10000
    P.loop.n_kt2 = 10000
    return P


def resonance_list(pp, proc):
    """Resonance names: the card's PROCESSPARAM RES list, replaced by an @RES{name:1, ...}
    command (MGraniitti::ReadProcessParam, src/MGraniitti.cc:456-477)."""
    names = list(pp.get("RES", []))
    for ident, _, args in split_commands(proc):
        if ident == "RES":
            names = [k for k, v in args.items() if v in ("true", "1")]
    return names


def set_resonances(P, pp, proc, tune, finals, allow_none=False, regge=False):
    """Resonance parameters (PARAM_RES), '@R[name]{M:.., W:.., gN:.., JZn:..}' overrides
    (src/MGraniitti.cc:480-575) and the decay couplings (MProcess::SetupBranching,
    src/MProcess.cc:471-520), in the order the reference applies them. With allow_none
    (RES+CONTENSOR, RES+CON) an empty list leaves the continuum alone (MSubProc.h:333).
    regge: the Regge model's coupling g_A exp(i g_phi), form factor, Breit-Wigner form,
    spin density matrix and decay coupling sqrt(BR W / Gamma_PS)."""
    table = RESONANCES.get(tune, {})
    names = resonance_list(pp, proc)
    if not names and allow_none:
        P.n_res = 0
        return
    if not names:
        raise ValueError("RESTENSOR needs resonances: PROCESSPARAM RES or @RES{name:1}")
    if len(names) > _abi.GRN_MAX_RESONANCES:
        raise UnsupportedProcess("at most %d resonances in the coherent sum"
                                 % _abi.GRN_MAX_RESONANCES)
    res = {}
    for n in names:
        if n not in table:
            raise UnsupportedProcess("resonance %s (decaying to %s) is not available"
                                     % (n, " ".join(finals)))
        res[n] = dict(table[n], g_Tensor=list(table[n]["g_Tensor"]))
        if "rho" in table[n]:
            res[n]["rho"] = list(table[n]["rho"])
    for ident, targets, args in split_commands(proc):
        if ident != "R":
            continue
        if len(targets) != 1 or targets[0] not in res:
            raise ValueError("@R[] needs one target among the resonances: %r" % targets)
        r = res[targets[0]]
        # JZn: diagonal spin density entries of M = +-n, then normalised to unit trace
        jz = {int(k[2:]): float(v) for k, v in args.items() if k.startswith("JZ") and k[2:].isdigit()}
        if jz and r["J"] != 0:
            J = r["J"]
            diag = [0.0] * (2 * J + 1)
            for n_, v in jz.items():
                if v < 0:
                    raise ValueError("@R[] JZ value < 0")
                if n_ <= J:
                    diag[J - n_] = diag[J + n_] = v
            tr = sum(diag)
            if not tr > 0:
                raise ValueError("@R[] spin density with zero trace")
            r["rho"] = [d / tr for d in diag]
        for k, v in args.items():
            if k == "M":
                r["M"] = float(v)
            elif k == "W":
                r["W"] = float(v)
            elif k.startswith("g") and k[1:].isdigit() and int(k[1:]) < len(r["g_Tensor"]):
                r["g_Tensor"][int(k[1:])] = float(v)
    lib = _abi.load_library()
    pair = tuple(sorted(finals))  # ("pi+", "pi-"), ("K+", "K-")
    P.n_res = len(names)
    for i, n in enumerate(names):
        r = res[n]
        br = BRANCHING.get(r["pdg"], {}).get(pair)
        if br is None:
            raise UnsupportedProcess("no branching ratio for %s -> %s" % (n, " ".join(finals)))
        R = P.res[i]
        R.J, R.P, R.M, R.W = r["J"], r["P"], r["M"], r["W"]
        for k, g in enumerate(r["g_Tensor"]):
            R.g_tensor[k] = g
        if regge:
            R.g_decay = lib.grn_regge_decay_coupling(r["M"], r["W"], PARTICLES[finals[0]][1], br)
            R.g_regge[0] = r["g_A"] * math.cos(r["g_phi"])
            R.g_regge[1] = r["g_A"] * math.sin(r["g_phi"])
            R.g_ff, R.bw = r["g_FF"], r["BW"]
            if r["J"] == 2:
                for m_, d in enumerate(r["rho"]):
                    R.rho[0][6 * m_] = d
        else:
            R.g_decay = lib.grn_tensor_decay_coupling(r["J"], r["M"], r["W"],
                                                      PARTICLES[finals[0]][1], br)


def vegas_params(card, prec=_abi.GRN_PREC_FP64, seed=1):
    v = card.get("INTEGRALPARAM", {}).get("VEGAS", {})
    vp = _abi.VegasParams()
    vp.bins = int(v.get("BINS", 128))
    if vp.bins % 2:
        raise ValueError("VEGAS::BINS must be even")
    vp.iter = int(v.get("ITER", 15))
    vp.ncall = int(v.get("NCALL", 20000))
    vp.lambda_ = float(v.get("LAMBDA", 1.5))
    vp.chi2max = float(v.get("CHI2MAX", 10.0))
    vp.precision = float(v.get("PRECISION", 0.01))
    vp.burnin_iter = 3
    vp.prec = prec
    vp.seed = seed
    return vp

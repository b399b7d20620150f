"""Steering-card parsing and parameter derivation (host logic)."""
import pytest

from conftest import CARD, CARD_SCR
from graniitti_gb300 import card


def test_parse_process():
    i, c, k, f, o = card.parse_process("PP[CON]<C> -> pi+ pi- @OFFSHELL:0")
    assert (i, c, k, f) == ("PP", "CON", "C", ["pi+", "pi-"]) and o == {"OFFSHELL": "0"}


def test_json5_comments_and_trailing_commas():
    s = '{ // c\n "a": [1, 2,], /* x */ "b": "//not a comment", }'
    import json
    assert json.loads(card.strip_json5(s)) == {"a": [1, 2], "b": "//not a comment"}


def test_params_from_card():
    P = card.build_params(card.read_card(CARD))
    assert P.sqrt_s == 13000.0 and P.screening == 0 and P.n_central == 2
    assert abs(P.m_central[0] - 0.13957061) < 1e-12 and P.s_factor == 1.0
    assert (P.gcuts.rap_min, P.gcuts.rap_max, P.gcuts.kt_max, P.gcuts.fpt_max) == (-0.9, 0.9, 5.0, 2.5)
    assert P.fcuts.active == 1 and P.fcuts.pt_min == 0.1 and P.fcuts.eta_max == 0.9
    assert P.regge.offshellFF == 2 and abs(P.regge.c[0] - 35.00184) < 1e-12
    assert list(P.regge.active) == [1, 0, 0]
    assert (P.loop.n_kt, P.loop.n_phi, P.loop.kt_max) == (15, 12, 1.75)
    Ps = card.build_params(card.read_card(CARD_SCR))
    assert Ps.screening == 1


def test_identical_particles_symmetry_factor():
    P = card.build_params(card.read_card(CARD), "PP[CON]<C> -> pi0 pi0")
    assert P.s_factor == 2.0


def test_factorized_params():
    P = card.build_params(card.read_card(CARD), "PP[CON]<F> -> pi+ pi-")
    assert P.phase_space == 2 and (P.gcuts.Y_min, P.gcuts.Y_max) == (-0.9, 0.9)
    assert (P.gcuts.M_min, P.gcuts.M_max) == (0.0, 5.0)


def test_tensor_params():
    P = card.build_params(card.read_card(CARD), "PP[CONTENSOR]<C> -> pi+ pi-")
    assert P.process == 2 and P.tensor.gPps == 1.76 and P.tensor.em_kelly == 1
    PK = card.build_params(card.read_card(CARD), "PP[CONTENSOR]<C> -> K+ K-")
    assert PK.tensor.gPps == 1.54


def test_split_commands():
    cmds = card.split_commands("PP[RESTENSOR]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:true} "
                               "@R[f2_1270]{g0:1.5, M:1.3} @OFFSHELL:0 @FLAG")
    assert cmds == [("RES", [], {"f0_980": "1", "f2_1270": "true"}),
                    ("R", ["f2_1270"], {"g0": "1.5", "M": "1.3"}),
                    ("OFFSHELL", [], {"_SINGLET_": "0"}), ("FLAG", [], {"_SINGLET_": "true"})]
    with pytest.raises(ValueError):
        card.split_commands("X -> a b @R[f2{g0:1}")


# Decay couplings the reference prints for these resonances ("Tensor Pomeron decay
# couplings", MProcess::ProcessHelicityDecay): f2(1270) -> pi+ pi- 9.285, f0(980) -> pi+ pi-
# 1.434, f0(980) -> K+ K- 2.010 (below threshold: taken at M + W), f2(1270) -> K+ K- 5.503,
# f2 with @R{M:1.3, W:0.2} -> pi+ pi- 9.317.
def test_resonance_params_and_decay_couplings(lib_built):
    from conftest import GOLDEN
    import os
    c = card.read_card(os.path.join(GOLDEN, "cards", "pp_res_pipi.json"))
    P = card.build_params(c)
    assert P.process == 3 and P.phase_space == 2 and P.n_res == 1
    r = P.res[0]
    assert (r.J, r.P, r.M, r.W, r.g_tensor[0]) == (2, 1, 1.2755, 0.1867, 2.0)
    assert round(r.g_decay, 3) == 9.285
    P = card.build_params(c, "PP[RESTENSOR]<F> -> K+ K- @RES{f0_980:1, f2_1270:1}")
    assert [round(P.res[i].g_decay, 3) for i in range(2)] == [2.010, 5.503]
    P = card.build_params(c, "PP[RESTENSOR]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1} "
                             "@R[f2_1270]{M:1.3, W:0.2, g0:1.5}")
    assert [round(P.res[i].g_decay, 3) for i in range(2)] == [1.434, 9.317]
    assert (P.res[1].M, P.res[1].W, P.res[1].g_tensor[0]) == (1.3, 0.2, 1.5)
    assert (P.res[0].J, P.res[0].g_tensor[0], P.res[0].g_tensor[1]) == (0, 0.4, 2.0)
    from graniitti_gb300 import _abi
    lib = _abi.load_library()
    assert lib.grn_tensor_decay_coupling(4, 2.6, 0.1, 0.14, 1.0) == 1.0
    assert lib.grn_tensor_decay_coupling(3, 2.6, 0.1, 0.14, 1.0) != \
        lib.grn_tensor_decay_coupling(3, 2.6, 0.1, 0.14, 1.0)  # NaN


def test_resonances_plus_continuum_params(lib_built):
    from conftest import GOLDEN
    import os
    from graniitti_gb300 import _abi
    c = card.read_card(os.path.join(GOLDEN, "cards", "pp_res_pipi.json"))
    P = card.build_params(c, "PP[RES+CONTENSOR]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1}")
    assert P.process == _abi.GRN_PROC_TENSOR_RESCON and P.n_res == 2
    assert P.tensor.gPps == 1.76 and round(P.res[1].g_decay, 3) == 9.285
    c["PROCESSPARAM"]["RES"] = []
    P = card.build_params(c, "PP[RES+CONTENSOR]<C> -> K+ K-")  # the continuum alone
    assert P.n_res == 0 and P.tensor.gPps == 1.54
    with pytest.raises(ValueError):
        card.build_params(c, "PP[RESTENSOR]<C> -> K+ K-")


@pytest.mark.parametrize("proc", [
    "PP[RESTENSOR]<F> -> pi+ pi- @RES{rho_770:1}",       # no pseudoscalar-pair resonance
    "PP[RESTENSOR]<F> -> pi0 pi0 @RES{f2_1270:1}",
    "PP[RESTENSOR]<F> -> pi+ pi- @RES{f0_500:1, f0_980:1, f0_1500:1, f0_1710:1, f2_1270:1}"])
def test_unsupported_resonances_are_rejected(lib_built, proc):
    from conftest import GOLDEN
    import os
    c = card.read_card(os.path.join(GOLDEN, "cards", "pp_res_pipi.json"))
    with pytest.raises(card.UnsupportedProcess):
        card.build_params(c, proc)


def test_regge_resonance_params(lib_built):
    from conftest import GOLDEN
    import os
    from graniitti_gb300 import _abi
    c = card.read_card(os.path.join(GOLDEN, "cards", "pp_res_pipi.json"))
    P = card.build_params(c, "PP[RES+CON]<F> -> pi+ pi- @RES{f0_980:1, f2_1270:1} @FRAME:HX "
                             "@SPINDEC:false @R[f2_1270]{JZ0:1, JZ2:1}")
    assert P.process == _abi.GRN_PROC_REGGE_RESCON and P.n_res == 2
    assert (P.spin_gen, P.spin_dec, P.spin_frame, P.omega) == (1, 0, _abi.GRN_FRAME_HX, 0.5)
    f0, f2 = P.res[0], P.res[1]
    assert (f0.bw, f0.g_ff) == (2, 1.0) and abs(f0.g_regge[0] + 0.065) < 1e-6
    assert abs(complex(f2.g_regge[0], f2.g_regge[1]) - 0.7j * -1) < 1e-3  # 0.7 exp(-1.57 i)
    assert [f2.rho[0][6 * m] for m in range(5)] == [1 / 3, 0, 1 / 3, 0, 1 / 3]
    # sqrt(BR W / Gamma_PS): f2(1270) -> pi+ pi-, BR 0.562
    assert abs(f2.g_decay - 2.6257) < 1e-3
    P = card.build_params(c, "PP[RES]<C> -> K+ K- @RES{f0_980:1}")  # f0(980) below threshold
    assert P.process == _abi.GRN_PROC_REGGE_RES and P.n_res == 1 and P.spin_frame == 2
    with pytest.raises(card.UnsupportedProcess):
        card.build_params(c, "PP[RES]<C> -> pi+ pi- @FRAME:GJ")


@pytest.mark.parametrize("proc", ["PP[RESHEL]<C> -> pi+ pi-", "PP[CON]<Q> -> pi+ pi-",
                                  "PP[CON]<C> -> pi+ pi- pi+ pi- pi+", "yy[CON]<C> -> mu+ mu-",
                                  "PP[CONTENSOR]<F> -> pi+ pi- pi+ pi-",
                                  "PP[CON]<C> -> pi+ pi- pi+ pi- pi+ pi- pi+ pi-"])
def test_unsupported_processes_are_rejected(proc):
    with pytest.raises(card.UnsupportedProcess):
        card.build_params(card.read_card(CARD), proc)


def test_six_body_continuum():
    """PP[CON]<C|F> -> 6 bodies (MRegge::ME8): 20 hypercube dimensions, the continuum class's
    default kt_max = 10 GeV / 6 (MContinuum.cc:72-77)."""
    for cls in ("C", "F"):
        P = card.build_params(card.read_card(CARD), "PP[CON]<%s> -> pi+ pi- pi+ pi- pi+ pi-" % cls)
        assert P.n_central == 6 and P.process == card._abi.GRN_PROC_REGGE_CON
        assert P.s_factor == 36.0  # 3! 3!
        if cls == "C":
            assert abs(P.gcuts.kt_max - 10.0 / 6) < 1e-15


def test_vegas_params():
    vp = card.vegas_params(card.read_card(CARD))
    assert (vp.bins, vp.ncall, vp.iter, vp.lambda_, vp.precision) == (128, 100000, 5, 1.5, 0.001)


def test_offshell_command_and_continuum_cascades():
    """@OFFSHELL:x sets the widths of the cascades' Breit-Wigner draws (MProcess::SetOFFSHELL);
    the continuum class <C> takes two-body cascades of both central particles."""
    from graniitti_gb300 import _abi
    rr = "rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-}"
    c = card.read_card(CARD)
    P = card.build_params(c, "PP[CONTENSOR]<C> -> " + rr + " @OFFSHELL:0")
    assert P.phase_space == _abi.GRN_PS_CONTINUUM and P.n_decay == 2 and P.central_spin == 1
    assert (P.offshell_user, P.offshell) == (1, 0.0)
    P = card.build_params(c, "PP[CON]<F> -> " + rr + " @OFFSHELL:2.5")
    assert (P.offshell_user, P.offshell) == (1, 2.5)
    P = card.build_params(c, "PP[CONTENSOR]<C> -> " + rr)
    assert P.offshell_user == 0  # the reference default, 5 widths

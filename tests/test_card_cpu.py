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


@pytest.mark.parametrize("proc", ["PP[RES]<C> -> pi+ pi-", "PP[CON]<Q> -> pi+ pi-",
                                  "PP[CON]<C> -> pi+ pi- pi+ pi-", "yy[CON]<C> -> mu+ mu-"])
def test_unsupported_processes_are_rejected(proc):
    with pytest.raises(card.UnsupportedProcess):
        card.build_params(card.read_card(CARD), proc)


def test_vegas_params():
    vp = card.vegas_params(card.read_card(CARD))
    assert (vp.bins, vp.ncall, vp.iter, vp.lambda_, vp.precision) == (128, 100000, 5, 1.5, 0.001)

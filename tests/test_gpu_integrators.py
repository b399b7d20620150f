"""The three integrators of the generator's cards (INTEGRATOR VEGAS / FLAT / NEURO) through
the MGraniitti-style driver: same cross section within the combined statistical errors,
generation of unweighted events from VEGAS and from the flow."""
import json
import os

import numpy as np
import pytest

from conftest import CARD

pytestmark = pytest.mark.gpu


def _card(tmp_path, integrator, **vegas):
    from graniitti_gb300 import card
    c = card.read_card(CARD)
    c["GENERALPARAM"]["INTEGRATOR"] = integrator
    c["INTEGRALPARAM"]["VEGAS"].update({"NCALL": 1 << 18, "PRECISION": 2e-3}, **vegas)
    c["INTEGRALPARAM"]["FLAT"] = {"PRECISION": 3e-3, "MIN_EVENTS": 1 << 20}
    c["INTEGRALPARAM"]["FLOW"] = {"NTRAIN": 1 << 19, "BATCH": 16384, "EPOCHS": 4, "MIX": 0.05}
    p = os.path.join(str(tmp_path), "card_%s.json" % integrator)
    json.dump(c, open(p, "w"))
    return p


@pytest.fixture(scope="module")
def vegas_xs(gpu, tmp_path_factory):
    import graniitti_gb300 as g
    gen = g.Graniitti()
    gen.ReadInput(_card(tmp_path_factory.mktemp("v"), "VEGAS"))
    gen.Initialize()
    return gen.GetXS()


def test_flat_matches_vegas(gpu, tmp_path, vegas_xs):
    import graniitti_gb300 as g
    gen = g.Graniitti()
    gen.ReadInput(_card(tmp_path, "FLAT"))
    r = gen.Initialize()
    s, e = gen.GetXS()
    assert e / s < 3e-3 and r.evaluations >= 1 << 20
    pull = (s - vegas_xs[0]) / np.hypot(e, vegas_xs[1])
    print("FLAT %.6e +- %.1e (%d passes) vs VEGAS %.6e +- %.1e: pull %.2f"
          % (s, e, r.iterations, vegas_xs[0], vegas_xs[1], pull))
    assert abs(pull) < 4
    assert gen.GetMaxweight() > 0


def test_neuro_matches_vegas_and_generates(gpu, tmp_path, vegas_xs):
    import graniitti_gb300 as g
    gen = g.Graniitti()
    gen.ReadInput(_card(tmp_path, "NEURO"))
    gen.Initialize()
    s, e = gen.GetXS()
    pull = (s - vegas_xs[0]) / np.hypot(e, vegas_xs[1])
    tr = gen.train_result
    print("NEURO %.6e +- %.1e vs VEGAS: pull %.2f; training rel var %.3f -> %.3f"
          % (s, e, pull, tr.rel_var_start, tr.rel_var_flow))
    assert abs(pull) < 4 and tr.rel_var_flow < tr.rel_var_start
    pts, trials, ovf = gen.Generate(2000)
    assert pts.shape == (2000, 8) and trials >= 2000
    w, _ = gen.engine.event_weights(pts)
    assert np.all(w > 0)


def test_unknown_integrator_rejected(tmp_path):
    import graniitti_gb300 as g
    p = _card(tmp_path, "MCMC")
    gen = g.Graniitti()
    with pytest.raises(ValueError):
        gen.ReadInput(p)


def test_generated_events_written_as_records(gpu, tmp_path):
    """Generation with an output file: records of the accepted points, momentum conserved,
    central pions inside the fiducial cuts of the card, cross section in pb."""
    import graniitti_gb300 as g
    from graniitti_gb300.record import read_hepmc3
    gen = g.Graniitti()
    gen.ReadInput(_card(tmp_path, "VEGAS"))
    gen.Initialize()
    out = str(tmp_path / "events.hepmc3")
    pts, trials, ovf = gen.Generate(300, output=out)
    ev = read_hepmc3(out)
    assert len(ev) == 300
    s, e = gen.GetXS()
    for k in range(300):
        P = ev[k]["particles"]
        assert ev[k]["xs"][0] == pytest.approx(s * 1e12, rel=1e-15)
        p = {i: P[i][2] for i in P}
        tot = p[2] + p[5] + p[8] + p[9]
        assert np.allclose(tot, p[1] + p[4], atol=1e-8 * 13000)
        for i in (8, 9):
            px, py, pz, E = p[i]
            pt = np.hypot(px, py)
            eta = np.arcsinh(pz / pt)
            assert abs(eta) < 0.9 and pt > 0.1
        assert sorted([P[8][1], P[9][1]]) == [-211, 211]

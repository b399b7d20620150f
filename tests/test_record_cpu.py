"""Event-record writer (grn_write_records) on the CPU: the three formats carry the
record layout of MProcess::CommonRecord with 4-momentum conserved at every vertex."""
import numpy as np
import pytest

SQRT_S, MP, MPI = 13000.0, 0.938272081, 0.13957061


def _events(n, seed=1):
    """Synthetic exclusive events with exact 4-momentum conservation."""
    rng = np.random.default_rng(seed)
    Eb = SQRT_S / 2
    pzb = np.sqrt(Eb * Eb - MP * MP)
    out = np.zeros((n, 4, 4))
    for i in range(n):
        pt1, pt2 = rng.uniform(0.05, 0.8, 2)
        f1, f2 = rng.uniform(0, 2 * np.pi, 2)
        x1, x2 = rng.uniform(1e-5, 1e-3, 2)
        p1 = np.array([pt1 * np.cos(f1), pt1 * np.sin(f1), pzb * (1 - x1), 0.0])
        p2 = np.array([pt2 * np.cos(f2), pt2 * np.sin(f2), -pzb * (1 - x2), 0.0])
        p1[3] = np.sqrt(MP * MP + p1[:3] @ p1[:3])
        p2[3] = np.sqrt(MP * MP + p2[:3] @ p2[:3])
        X = np.array([0, 0, 0, SQRT_S]) - p1 - p2
        # split X into two pions isotropically in its rest frame
        M = np.sqrt(X[3] ** 2 - X[:3] @ X[:3])
        pst = np.sqrt(M * M / 4 - MPI * MPI)
        ct, ph = rng.uniform(-1, 1), rng.uniform(0, 2 * np.pi)
        st = np.sqrt(1 - ct * ct)
        k = np.array([pst * st * np.cos(ph), pst * st * np.sin(ph), pst * ct, M / 2])
        b = X[:3] / X[3]
        g = X[3] / M
        def boost(v):
            bp = b @ v[:3]
            e = g * (v[3] + bp)
            p = v[:3] + ((g - 1) * bp / (b @ b) + g * v[3]) * b
            return np.array([p[0], p[1], p[2], e])
        a = boost(k)
        kb = k.copy(); kb[:3] *= -1
        c = boost(kb)
        out[i] = [p1, p2, a, c]
    return out


@pytest.mark.parametrize("fmt", ["hepmc3", "hepmc2", "hepevt"])
def test_records_round_trip(tmp_path, fmt):
    from graniitti_gb300.record import EventWriter, read_hepmc3
    p4 = _events(20)
    path = str(tmp_path / ("ev." + fmt))
    with EventWriter(path, fmt, card="card.json") as w:
        w.write_momenta(p4, [2212, 211, -211], [MP, MPI, MPI], SQRT_S, 1.65e7, 6.3e3)
    text = open(path).read()
    if fmt == "hepmc3":
        assert text.startswith("HepMC::Version 3") and "Asciiv3-END_EVENT_LISTING" in text
        ev = read_hepmc3(path)
        assert len(ev) == 20
        for k, e in enumerate(ev):
            P = e["particles"]
            assert e["nv"] == 4 and e["np"] == 9 and len(P) == 9
            assert e["weights"] == [1.0] and e["xs"] == (1.65e7, 6.3e3)
            assert [P[i][1] for i in range(1, 10)] == [2212, 2212, 99, 2212, 2212, 99, 90, 211, -211]
            assert [P[i][4] for i in range(1, 10)] == [4, 1, 81, 4, 1, 81, 81, 1, 1]
            assert e["vertices"] == {-3: [3, 6]}
            p = {i: P[i][2] for i in P}
            scale = SQRT_S
            assert np.allclose(p[1], p[2] + p[3], atol=1e-9 * scale)       # v1
            assert np.allclose(p[4], p[5] + p[6], atol=1e-9 * scale)       # v2
            assert np.allclose(p[3] + p[6], p[7], atol=1e-7 * scale)       # v3
            assert np.allclose(p[7], p[8] + p[9], atol=1e-9 * scale)       # v4
            assert np.allclose(p[8], p4[k, 2], rtol=1e-15, atol=0)
    elif fmt == "hepmc2":
        assert "IO_GenEvent-START_EVENT_LISTING" in text and text.count("\nE ") == 20
        assert text.count("\nV ") == 80 and text.count("\nP ") == 180
    else:
        lines = text.strip().split("\n")
        assert len(lines) == 20 * 10 and lines[0].split()[:2] == ["E", "0"]
        row = lines[1].split()
        assert int(row[0]) == 4 and int(row[1]) == 2212 and int(row[4]) == 2 and int(row[5]) == 3


def test_writer_rejects_bad_format(tmp_path):
    from graniitti_gb300.record import EventWriter
    with pytest.raises(ValueError):
        EventWriter(str(tmp_path / "x"), "lhe")


def _boost(v, P):
    """Boost v (px, py, pz, E) from the rest frame of P to the frame of P."""
    M = np.sqrt(P[3] ** 2 - P[:3] @ P[:3])
    b = P[:3] / P[3]
    g = P[3] / M
    bp = b @ v[:3]
    e = g * (v[3] + bp)
    p = v[:3] + (((g - 1) * bp / (b @ b) if b @ b > 0 else 0.0) + g * v[3]) * b
    return np.array([p[0], p[1], p[2], e])


def _decay(P, m, rng):
    M = np.sqrt(P[3] ** 2 - P[:3] @ P[:3])
    pst = np.sqrt(M * M / 4 - m * m)
    ct, ph = rng.uniform(-1, 1), rng.uniform(0, 2 * np.pi)
    st = np.sqrt(1 - ct * ct)
    k = np.array([pst * st * np.cos(ph), pst * st * np.sin(ph), pst * ct, M / 2])
    kb = k.copy()
    kb[:3] *= -1
    return _boost(k, P), _boost(kb, P)


@pytest.mark.parametrize("fmt", ["hepmc3", "hepmc2", "hepevt"])
def test_cascade_records(tmp_path, fmt):
    """rho rho -> pi+ pi- pi+ pi- records: the central particles with status 2 and their decay
    vertices (WriteDecayKinematics), four-momentum conserved at all six vertices."""
    from graniitti_gb300.record import EventWriter, read_hepmc3
    rng = np.random.default_rng(3)
    p4 = _events(200, seed=2)
    mX = np.sqrt(np.maximum(0, (p4[:, 2, 3] + p4[:, 3, 3]) ** 2 -
                            ((p4[:, 2, :3] + p4[:, 3, :3]) ** 2).sum(axis=1)))
    p4 = p4[mX > 1.7][:10].copy()  # central systems heavy enough for two 0.78 GeV states
    assert len(p4) == 10
    pd = np.zeros((10, 4, 4))
    for i in range(10):
        X = p4[i, 2] + p4[i, 3]
        r1, r2 = _decay(X, 0.78, rng)  # the central pair as two off-shell vector mesons
        p4[i, 2], p4[i, 3] = r1, r2
        pd[i, 0], pd[i, 1] = _decay(r1, MPI, rng)
        pd[i, 2], pd[i, 3] = _decay(r2, MPI, rng)
    path = str(tmp_path / ("cas." + fmt))
    with EventWriter(path, fmt) as w:
        w.write_cascade_momenta(p4, pd, [2212, 113, 113, 211, -211, 211, -211],
                                [MP, 0.77526, 0.77526, MPI, MPI, MPI, MPI], SQRT_S, 1e3, 10.0)
    text = open(path).read()
    if fmt == "hepmc3":
        ev = read_hepmc3(path)
        assert len(ev) == 10
        for k, e in enumerate(ev):
            P = e["particles"]
            assert e["nv"] == 6 and e["np"] == 13 and len(P) == 13
            assert [P[i][1] for i in range(1, 14)] == [2212, 2212, 99, 2212, 2212, 99, 90, 113,
                                                      113, 211, -211, 211, -211]
            assert [P[i][4] for i in range(1, 14)] == [4, 1, 81, 4, 1, 81, 81, 2, 2, 1, 1, 1, 1]
            assert [P[i][0] for i in range(8, 14)] == [7, 7, 8, 8, 9, 9]
            p = {i: P[i][2] for i in P}
            assert np.allclose(p[7], p[8] + p[9], atol=1e-9 * SQRT_S)
            assert np.allclose(p[8], p[10] + p[11], atol=1e-12)
            assert np.allclose(p[9], p[12] + p[13], atol=1e-12)
            assert abs(P[8][3] - 0.78) < 1e-9  # off-shell mass of the central particle
    elif fmt == "hepmc2":
        assert text.count("\nE ") == 10 and text.count("\nV ") == 60 and text.count("\nP ") == 130
    else:
        lines = text.strip().split("\n")
        assert len(lines) == 10 * 14
        rows = [l.split() for l in lines[1:14]]
        assert [int(r[0]) for r in rows[7:9]] == [2, 2]
        assert [int(x) for x in rows[7][2:6]] == [7, 7, 10, 11]
        assert [int(x) for x in rows[12][2:6]] == [9, 9, 0, 0]

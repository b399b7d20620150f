"""Event records of accepted points: the output path of MGraniitti::SaveEvent.

EventWriter wraps the library's writer (grn_writer_open / grn_write_events /
grn_write_records): FORMAT "hepmc3", "hepmc2" or "hepevt" with the record layout of
MProcess::CommonRecord (src/MProcess.cc:1588-1680). read_hepmc3 parses the ASCII v3
files it writes (events as lists of particles and vertices), for checks and analysis.
"""
import ctypes

import numpy as np

from . import _abi


class EventWriter:
    def __init__(self, path, fmt="hepmc3", tool="GRANIITTI", card=None):
        self.lib = _abi.load_library()
        if fmt not in _abi.FORMATS:
            raise ValueError("MGraniitti::SaveEvent: Unknown output FORMAT %s" % fmt)
        h = ctypes.c_void_p()
        st = self.lib.grn_writer_open(path.encode(), _abi.FORMATS[fmt], tool.encode(),
                                      card.encode() if card else None, ctypes.byref(h))
        if st != _abi.GRN_OK:
            raise OSError("cannot open %s for writing" % path)
        self.h = h
        self.path = path
        self.written = 0

    def write_points(self, engine, u, pdg, sigma_pb, sigma_err_pb, weight=1.0):
        """Events of hypercube points u (n x dim): kinematics on the engine, then records.
        pdg: beam, the two central particles and, for cascades, the four daughters."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        pd = (ctypes.c_int32 * len(pdg))(*pdg)
        n = ctypes.c_int64()
        _abi.check(self.lib.grn_write_events(self.h, engine.h, u.ctypes.data_as(ctypes.c_void_p),
                                             u.shape[0], pd, len(pdg), weight, sigma_pb,
                                             sigma_err_pb, ctypes.byref(n)))
        self.written += n.value
        return n.value

    def write_momenta(self, p4, pdg, masses, sqrt_s, sigma_pb, sigma_err_pb, weight=1.0):
        """Events from 4-vectors (n x 4 x 4: forward 1, forward 2, central 1, central 2)."""
        p4 = np.ascontiguousarray(p4, dtype=np.float64)
        pd = (ctypes.c_int32 * 3)(*pdg)
        ms = (ctypes.c_double * 3)(*masses)
        _abi.check(self.lib.grn_write_records(self.h, p4.ctypes.data_as(ctypes.c_void_p),
                                              p4.shape[0], pd, ms, sqrt_s, weight, sigma_pb,
                                              sigma_err_pb))
        self.written += p4.shape[0]

    def write_cascade_momenta(self, p4, pd, pdg, masses, sqrt_s, sigma_pb, sigma_err_pb,
                              weight=1.0):
        """Cascade events from 4-vectors: p4 (n x 4 x 4) as for write_momenta with the
        central particles off shell, pd (n x 4 x 4) their four daughters; pdg, masses: beam,
        the two central particles, the four daughters."""
        p4 = np.ascontiguousarray(p4, dtype=np.float64)
        pd = np.ascontiguousarray(pd, dtype=np.float64)
        ids = (ctypes.c_int32 * 7)(*pdg)
        ms = (ctypes.c_double * 7)(*masses)
        _abi.check(self.lib.grn_write_cascade_records(
            self.h, p4.ctypes.data_as(ctypes.c_void_p), pd.ctypes.data_as(ctypes.c_void_p),
            p4.shape[0], ids, ms, sqrt_s, weight, sigma_pb, sigma_err_pb))
        self.written += p4.shape[0]

    def close(self):
        if getattr(self, "h", None):
            self.lib.grn_writer_close(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def read_hepmc3(path):
    """Events of a HepMC3 ASCII v3 file as dicts: weights, cross section, particles
    {id: (parent, pdg, p[4], m, status)} and vertices {id: [incoming particle ids]}."""
    events, ev = [], None
    with open(path) as f:
        for line in f:
            t = line.split()
            if not t:
                continue
            if t[0] == "E":
                ev = {"number": int(t[1]), "nv": int(t[2]), "np": int(t[3]), "particles": {},
                      "vertices": {}, "weights": [], "xs": None}
                events.append(ev)
            elif ev is None:
                continue
            elif t[0] == "W":
                ev["weights"] = [float(x) for x in t[1:]]
            elif t[0] == "A" and t[2] == "GenCrossSection":
                ev["xs"] = (float(t[3]), float(t[4]))
            elif t[0] == "V":
                ins = t[3].strip("[]")
                ev["vertices"][int(t[1])] = [int(x) for x in ins.split(",") if x]
            elif t[0] == "P":
                ev["particles"][int(t[1])] = (int(t[2]), int(t[3]),
                                              np.array([float(x) for x in t[4:8]]), float(t[8]),
                                              int(t[9]))
    return events

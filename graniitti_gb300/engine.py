"""Host-side mirror of the generator's process / driver interface over the C ABI.

Engine      one process on one GPU: event weights (MProcess::EventWeight in batch),
            eikonal tables (MEikonal), VEGAS primitives and unweighting.
Graniitti   the MGraniitti flow: ReadInput(card, process) -> Initialize() (eikonal
            tables when screening is on, VEGAS integration) -> GetXS() ->
            Generate(n) unweighted events.

Arrays are numpy (host) or anything exposing data_ptr() with a CUDA device
(torch tensors); host arrays are staged by the library.
"""
import ctypes

import numpy as np

from . import _abi
from . import card as _card

FP64 = _abi.GRN_PREC_FP64
MIXED = _abi.GRN_PREC_MIXED


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return ctypes.c_void_p(a.data_ptr())
    if not a.flags["C_CONTIGUOUS"]:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data_as(ctypes.c_void_p)


class Engine:
    def __init__(self, params, device=0):
        self.lib = _abi.load_library()
        self.params = params
        h = ctypes.c_void_p()
        _abi.check(self.lib.grn_create(ctypes.byref(params), device, ctypes.byref(h)))
        self.h = h
        self.dim = self.lib.grn_dim(h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.grn_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def stream(self):
        return self.lib.grn_engine_stream(self.h)

    # -- event weights ------------------------------------------------------
    def event_weights(self, u, prec=FP64, w=None, flags=None):
        if hasattr(u, "data_ptr"):
            n = u.shape[0]
            _abi.check(self.lib.grn_event_weights(self.h, _ptr(u), n, self.dim, _ptr(w),
                                                  _ptr(flags), prec))
            return w, flags
        u = np.ascontiguousarray(u, dtype=np.float64)
        n = u.shape[0]
        if u.shape[1] != self.dim:
            raise ValueError("u must have %d columns" % self.dim)
        w = np.zeros(n) if w is None else w
        flags = np.zeros(n, dtype=np.uint8) if flags is None else flags
        _abi.check(self.lib.grn_event_weights(self.h, _ptr(u), n, self.dim, _ptr(w), _ptr(flags),
                                              prec))
        return w, flags

    def event_daughters(self, u):
        """Cascade daughters (n, 4, 4), or the central particles of a 4- or 6-body state
        (n, 4, 4) / (n, 6, 4)."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        pd = np.zeros((u.shape[0], 6 if self.params.n_central == 6 else 4, 4))
        _abi.check(self.lib.grn_event_daughters(self.h, _ptr(u), u.shape[0], self.dim, _ptr(pd)))
        return pd

    def event_kinematics(self, u):
        u = np.ascontiguousarray(u, dtype=np.float64)
        n = u.shape[0]
        p4 = np.zeros((n, 4, 4))
        ts = np.zeros((n, 2))
        fl = np.zeros(n, dtype=np.uint8)
        _abi.check(self.lib.grn_event_kinematics(self.h, _ptr(u), n, self.dim, _ptr(p4), _ptr(ts),
                                                 _ptr(fl)))
        return p4, ts, fl

    def uniforms(self, seed, n, dim=None, first=0, stream=0):
        dim = dim or self.dim
        out = np.zeros((n, dim))
        _abi.check(self.lib.grn_uniforms(self.h, seed, stream, first, n, dim, _ptr(out)))
        return out

    # -- eikonal ------------------------------------------------------------
    def eikonal_build(self, n_bt=0, n_kt2=0):
        _abi.check(self.lib.grn_eikonal_build(self.h, n_bt, n_kt2))

    def eikonal_xs(self):
        t, e, i = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        _abi.check(self.lib.grn_eikonal_xs(self.h, ctypes.byref(t), ctypes.byref(e),
                                           ctypes.byref(i)))
        return t.value, e.value, i.value

    def eikonal_tables(self, n_bt, n_kt2):
        mbt = np.zeros((n_bt + 1, 3))
        msa = np.zeros((n_kt2 + 1, 3))
        _abi.check(self.lib.grn_eikonal_get(self.h, _ptr(mbt), _ptr(msa)))
        return mbt, msa

    def eikonal_set(self, mbt, msa):
        mbt = np.ascontiguousarray(mbt, dtype=np.float64)
        msa = np.ascontiguousarray(msa, dtype=np.float64)
        _abi.check(self.lib.grn_eikonal_set(self.h, mbt.shape[0] - 1, _ptr(mbt), msa.shape[0] - 1,
                                            _ptr(msa)))

    # -- VEGAS --------------------------------------------------------------
    def vegas_init(self, vp):
        self.vp = vp
        _abi.check(self.lib.grn_vegas_init(self.h, ctypes.byref(vp)))

    def vegas_iteration(self, mode=1, refine=True, iter_id=1):
        r = _abi.VegasResult()
        _abi.check(self.lib.grn_vegas_iteration(self.h, mode, 1 if refine else 0, iter_id,
                                                ctypes.byref(r)))
        return r

    def vegas_integrate(self, vp):
        self.vp = vp
        r = _abi.VegasResult()
        _abi.check(self.lib.grn_vegas_integrate(self.h, ctypes.byref(vp), ctypes.byref(r)))
        return r

    def flat_integrate(self, ncall=1 << 20, precision=0.05, min_events=1000000, prec=FP64,
                       seed=1):
        fp = _abi.FlatParams(ncall=ncall, precision=precision, min_events=min_events, prec=prec,
                             seed=seed)
        r = _abi.VegasResult()
        _abi.check(self.lib.grn_flat_integrate(self.h, ctypes.byref(fp), ctypes.byref(r)))
        return r

    def vegas_clear(self):
        _abi.check(self.lib.grn_vegas_clear(self.h))

    def tuning(self):
        t = _abi.Tuning()
        _abi.check(self.lib.grn_get_tuning(self.h, ctypes.byref(t)))
        return t

    def set_tuning(self, loop_pair=None, vegas_blocks=None, weight_blocks=None,
                   fp64_refine=None, refine_tol=None, born_blocks=None, generic_blocks=None):
        t = self.tuning()
        if born_blocks is not None:
            t.born_blocks = int(born_blocks)
        if generic_blocks is not None:
            t.generic_blocks = int(generic_blocks)
        if fp64_refine is not None:
            t.fp64_refine = int(fp64_refine)
        if refine_tol is not None:
            t.refine_tol = float(refine_tol)
        if loop_pair is not None:
            t.loop_pair = loop_pair
        if vegas_blocks is not None:
            t.vegas_blocks = vegas_blocks
        if weight_blocks is not None:
            t.weight_blocks = weight_blocks
        _abi.check(self.lib.grn_set_tuning(self.h, ctypes.byref(t)))

    def autotune(self, sample=1 << 18):
        r = _abi.TuneResult()
        _abi.check(self.lib.grn_autotune(self.h, sample, ctypes.byref(r)))
        return r

    def get_maxweight(self):
        m = ctypes.c_double()
        _abi.check(self.lib.grn_get_maxweight(self.h, ctypes.byref(m)))
        return m.value

    def set_maxweight(self, maxf):
        _abi.check(self.lib.grn_set_maxweight(self.h, maxf))

    def vegas_grid(self):
        x = np.zeros((self.vp.bins, self.dim))
        _abi.check(self.lib.grn_vegas_get_grid(self.h, _ptr(x)))
        return x

    def vegas_set_grid(self, xmat):
        xmat = np.ascontiguousarray(xmat, dtype=np.float64)
        _abi.check(self.lib.grn_vegas_set_grid(self.h, _ptr(xmat)))

    def unweight(self, fmax, seed=7, cap=0):
        na, no = ctypes.c_int64(), ctypes.c_int64()
        idx = np.zeros(max(cap, 1), dtype=np.int64)
        _abi.check(self.lib.grn_unweight(self.h, fmax, seed, ctypes.byref(na), ctypes.byref(no),
                                         _ptr(idx) if cap > 0 else None, cap))
        return na.value, no.value, idx[:min(na.value, cap)]

    def vegas_points(self, idx):
        idx = np.ascontiguousarray(idx, dtype=np.int64)
        out = np.zeros((idx.shape[0], self.dim))
        _abi.check(self.lib.grn_vegas_points(self.h, _ptr(idx), idx.shape[0], _ptr(out)))
        return out

    def pass_weights(self, n):
        """f of every point of the last iteration (n = its ncall)."""
        f = np.zeros(n)
        _abi.check(self.lib.grn_pass_weights(self.h, _ptr(f), n))
        return f

    # On-the-fly histograms: specs are (obs, nbins, lo, hi) or
    # (obs, nbins, lo, hi, obs2, nbins2, lo2, hi2) with obs a name of _abi.OBS.
    def hist_define(self, specs):
        arr = (_abi.HistSpec * max(len(specs), 1))()
        self.hist_shapes = []
        for k, s in enumerate(specs):
            a = arr[k]
            a.obs, a.nbins, a.lo, a.hi = _abi.OBS.index(s[0]), s[1], s[2], s[3]
            if len(s) > 4:
                a.obs2, a.nbins2, a.lo2, a.hi2 = _abi.OBS.index(s[4]), s[5], s[6], s[7]
                self.hist_shapes.append((s[1], s[5]))
            else:
                self.hist_shapes.append((s[1],))
        _abi.check(self.lib.grn_hist_define(self.h, arr, len(specs)))

    def hist_fill(self):
        _abi.check(self.lib.grn_hist_fill(self.h))

    def hist_clear(self):
        _abi.check(self.lib.grn_hist_clear(self.h))

    def hist_get(self, h):
        """(sum of weights, sum of squared weights, fill counts, [below, above, NaN])."""
        shape = self.hist_shapes[h]
        nb = int(np.prod(shape))
        w, w2 = np.zeros(nb), np.zeros(nb)
        c, out = np.zeros(nb, dtype=np.int64), np.zeros(3, dtype=np.int64)
        _abi.check(self.lib.grn_hist_get(self.h, h, _ptr(w), _ptr(w2), _ptr(c), _ptr(out)))
        return w.reshape(shape), w2.reshape(shape), c.reshape(shape), out


class Flow:
    """Coupling-layer spline flow in front of the engine's VEGAS map (grn_flow_*).

    Point arrays are float32, dimension-major (dim x n)."""

    def __init__(self, engine, layers=6, seed=1, mix_uniform=0.0, hidden=128):
        self.engine = engine
        self.lib = engine.lib
        p = _abi.FlowParams()
        self.lib.grn_flow_default_params(ctypes.byref(p))
        p.dim = engine.dim
        p.hidden = hidden
        p.layers = layers
        p.seed = seed
        p.mix_uniform = mix_uniform
        h = ctypes.c_void_p()
        _abi.check(self.lib.grn_flow_create(engine.h, ctypes.byref(p), ctypes.byref(h)))
        self.h = h
        self.layers = layers
        self.hidden = hidden
        self.dim = engine.dim
        self.n_params = self.lib.grn_flow_num_params(h)

    def close(self):
        if getattr(self, "h", None):
            self.lib.grn_flow_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_wait_polls(self, polls):
        """Poll limit of the forward kernel's first bounded wait (< 0: the default); 0 makes
        the next forward call give up at once and fail with GRN_ERR_CUDA (diagnostic)."""
        _abi.check(self.lib.grn_flow_set_wait_polls(self.h, int(polls)))

    def get_params(self):
        t = np.zeros(self.n_params, dtype=np.float32)
        _abi.check(self.lib.grn_flow_get_params(self.h, _ptr(t)))
        return t

    def set_params(self, theta):
        t = np.ascontiguousarray(theta, dtype=np.float32)
        if t.shape != (self.n_params,):
            raise ValueError("expected %d parameters" % self.n_params)
        _abi.check(self.lib.grn_flow_set_params(self.h, _ptr(t)))

    def _pts(self, x):
        x = np.ascontiguousarray(x, dtype=np.float32)
        if x.ndim != 2 or x.shape[0] != self.dim:
            raise ValueError("points must be %d x n (dimension-major)" % self.dim)
        return x

    def density(self, x):
        x = self._pts(x)
        n = x.shape[1]
        z = np.zeros_like(x)
        lq = np.zeros(n, dtype=np.float32)
        _abi.check(self.lib.grn_flow_density(self.h, _ptr(x), n, _ptr(z), _ptr(lq)))
        return z, lq

    def inverse(self, z):
        z = self._pts(z)
        n = z.shape[1]
        x = np.zeros_like(z)
        lq = np.zeros(n, dtype=np.float32)
        _abi.check(self.lib.grn_flow_inverse(self.h, _ptr(z), n, _ptr(x), _ptr(lq)))
        return x, lq

    def sample(self, seed, n, stream=0, first=0):
        x = np.zeros((self.dim, n), dtype=np.float32)
        lq = np.zeros(n, dtype=np.float32)
        _abi.check(self.lib.grn_flow_sample(self.h, seed, stream, first, n, _ptr(x), _ptr(lq)))
        return x, lq

    def loss_grad(self, x, coef, kind=_abi.GRN_FLOW_LOSS_VARIANCE):
        x = self._pts(x)
        coef = np.ascontiguousarray(coef, dtype=np.float32)
        g = np.zeros(self.n_params, dtype=np.float32)
        loss = ctypes.c_double()
        _abi.check(self.lib.grn_flow_loss_grad(self.h, _ptr(x), _ptr(coef), x.shape[1], kind,
                                               ctypes.byref(loss), _ptr(g)))
        return loss.value, g

    def train_step(self, x, coef, lr=1e-3, kind=_abi.GRN_FLOW_LOSS_VARIANCE):
        x = self._pts(x)
        coef = np.ascontiguousarray(coef, dtype=np.float32)
        loss = ctypes.c_double()
        _abi.check(self.lib.grn_flow_train_step(self.h, _ptr(x), _ptr(coef), x.shape[1], kind,
                                                lr, ctypes.byref(loss)))
        return loss.value

    def train(self, n_train=1 << 22, batch=65536, epochs=4, rounds=1, lr=1e-3,
              loss=_abi.GRN_FLOW_LOSS_VARIANCE, prec=FP64, seed_stream=1):
        tp = _abi.FlowTrainParams(n_train=n_train, batch=batch, epochs=epochs, rounds=rounds,
                                  lr=lr, loss=loss, prec=prec, seed_stream=seed_stream)
        r = _abi.FlowTrainResult()
        _abi.check(self.lib.grn_flow_train(self.engine.h, self.h, ctypes.byref(tp),
                                           ctypes.byref(r)))
        return r

    def iteration(self, mode=1, iter_id=1):
        r = _abi.VegasResult()
        _abi.check(self.lib.grn_flow_iteration(self.engine.h, self.h, mode, iter_id,
                                               ctypes.byref(r)))
        return r

    def integrate(self, vp):
        r = _abi.VegasResult()
        _abi.check(self.lib.grn_flow_integrate(self.engine.h, self.h, ctypes.byref(vp),
                                               ctypes.byref(r)))
        return r


class Batch:
    """Several engines (processes) run one pass together: fused stage launches replayed
    as a CUDA graph (grn_batch_*)."""

    def __init__(self, engines):
        self.lib = engines[0].lib
        self.engines = list(engines)
        arr = (ctypes.c_void_p * len(engines))(*[e.h.value for e in engines])
        h = ctypes.c_void_p()
        _abi.check(self.lib.grn_batch_create(arr, len(engines), ctypes.byref(h)))
        self.h = h

    def set_flow(self, index, flow):
        """Member `index` draws its points from `flow` (None: Philox points)."""
        _abi.check(self.lib.grn_batch_set_flow(self.h, index, flow.h if flow else None))

    def iteration(self, mode=1, refine=True, iter_id=1):
        res = (_abi.VegasResult * len(self.engines))()
        ms = ctypes.c_double()
        _abi.check(self.lib.grn_batch_iteration(self.h, mode, 1 if refine else 0, iter_id, res,
                                                ctypes.byref(ms)))
        return list(res), ms.value

    def close(self):
        if getattr(self, "h", None):
            self.lib.grn_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Graniitti:
    """MGraniitti-style driver (src/MGraniitti.cc) over the GPU engine.

    INTEGRATOR (GENERALPARAM, as in the generator's cards):
      "VEGAS"  SampleVegas: burn-in + integration iterations (grn_vegas_integrate)
      "FLAT"   SampleFlat: uniform points until FLAT::PRECISION and MIN_EVENTS
      "NEURO"  the learned proposal: VEGAS adapts the grid, the coupling-layer flow is
               trained in front of it, then integration and generation run through the
               flow (the reference's NEURO prototype, SampleNeuro, samples through its own
               small network). Optional card block INTEGRALPARAM.FLOW (an extension of the
               card format): LAYERS, NTRAIN, BATCH, EPOCHS, ROUNDS, LR, MIX.
    """

    FLOW_DEFAULTS = {"LAYERS": 6, "NTRAIN": 1 << 22, "BATCH": 16384, "EPOCHS": 3, "ROUNDS": 4,
                     "LR": 1e-3, "MIX": 0.05}

    def __init__(self, device=0):
        self.device = device
        self.engine = None
        self.card = None
        self.vp = None
        self.result = None
        self.prec = FP64
        self.integrator = "VEGAS"
        self.flow = None
        self.train_result = None

    def ReadInput(self, inputfile, cmd_PROCESS=None):
        self.card = _card.read_card(inputfile)
        self.process = cmd_PROCESS or self.card["PROCESSPARAM"]["PROCESS"]
        self.params = _card.build_params(self.card, cmd_PROCESS)
        self.vp = _card.vegas_params(self.card, prec=self.prec)
        self.integrator = self.card.get("GENERALPARAM", {}).get("INTEGRATOR", "VEGAS")
        if self.integrator not in ("VEGAS", "FLAT", "NEURO"):
            raise ValueError("MGraniitti::CallIntegrator: Unknown INTEGRATOR = %s "
                             "(use VEGAS, FLAT, NEURO)" % self.integrator)
        ip = self.card.get("INTEGRALPARAM", {})
        fl = ip.get("FLAT", {})
        self.flat = {"PRECISION": float(fl.get("PRECISION", 0.05)),
                     "MIN_EVENTS": int(fl.get("MIN_EVENTS", 1000000))}
        self.flowp = dict(self.FLOW_DEFAULTS, **ip.get("FLOW", {}))
        self.engine = Engine(self.params, self.device)

    def SetIntegrator(self, name):
        if name not in ("VEGAS", "FLAT", "NEURO"):
            raise ValueError("unknown integrator %s" % name)
        self.integrator = name

    def SetVegasParam(self, **kw):
        for k, v in kw.items():
            setattr(self.vp, "lambda_" if k == "LAMBDA" else k.lower(), v)

    def SetPrecision(self, prec):
        self.prec = prec
        if self.vp is not None:
            self.vp.prec = prec

    def Initialize(self):
        if self.params.screening:
            self.engine.eikonal_build()
            if self.vp.prec == MIXED:
                self.engine.autotune(sample=1 << 16)
        if self.integrator == "FLAT":
            self.result = self.engine.flat_integrate(
                ncall=int(self.vp.ncall), precision=self.flat["PRECISION"],
                min_events=self.flat["MIN_EVENTS"], prec=self.vp.prec, seed=self.vp.seed)
            return self.result
        self.result = self.engine.vegas_integrate(self.vp)
        if self.integrator == "NEURO":
            fp = self.flowp
            ntrain = int(fp["NTRAIN"]) // int(fp["BATCH"]) * int(fp["BATCH"])
            self.flow = Flow(self.engine, layers=int(fp["LAYERS"]), seed=int(self.vp.seed),
                             mix_uniform=float(fp["MIX"]))
            self.train_result = self.flow.train(
                n_train=ntrain, batch=int(fp["BATCH"]), epochs=int(fp["EPOCHS"]),
                rounds=int(fp["ROUNDS"]), lr=float(fp["LR"]), prec=self.vp.prec)
            self.result = self.flow.integrate(self.vp)
        return self.result

    def GetXS(self):
        return self.result.sigma, self.result.sigma_err

    def GetMaxweight(self):
        return self.engine.get_maxweight()

    def Generate(self, nevents, seed=11, max_iter=1000, output=None, fmt=None):
        """Unweighted events: generation-mode passes (frozen grid, through the flow for
        NEURO) with hit-or-miss against the integration's max weight
        (MGraniitti.cc:1131-1134, 1651-1664). Returns (points, n_trials, n_overflow).
        With `output` (a path) the events are also written as event records in FORMAT
        (`fmt`, default the card's GENERALPARAM FORMAT), weight 1, cross section in pb."""
        if self.integrator == "FLAT":
            raise NotImplementedError("generation from FLAT integration is not provided")
        writer = None
        if output is not None:
            from .record import EventWriter
            fmt = fmt or self.card.get("GENERALPARAM", {}).get("FORMAT", "hepmc3")
            writer = EventWriter(output, fmt, tool="GRANIITTI (%s)" %
                                 self.card.get("GENERALPARAM", {}).get("MODELPARAM", "TUNE0"))
        fmax = self.engine.get_maxweight()
        pts, trials, ovf = [], 0, 0
        it = 0
        while sum(len(p) for p in pts) < nevents and it < max_iter:
            if self.integrator == "NEURO":
                self.flow.iteration(mode=2, iter_id=0x40000000 + it)
            else:
                self.engine.vegas_iteration(mode=2, refine=False, iter_id=0x40000000 + it)
            cap = int(self.vp.ncall)
            na, no, idx = self.engine.unweight(fmax, seed=seed + it, cap=cap)
            need = nevents - sum(len(p) for p in pts)
            idx = idx[:need]
            pts.append(self.engine.vegas_points(idx))
            trials += int(self.vp.ncall) if need >= na else int(idx[-1]) + 1
            ovf += no
            it += 1
        out = np.concatenate(pts) if pts else np.zeros((0, self.engine.dim))
        if writer is not None:
            pdg = self.card_pdg()
            writer.write_points(self.engine, out, pdg, self.result.sigma * 1e12,
                                self.result.sigma_err * 1e12)
            writer.close()
        return out, trials, ovf

    def card_pdg(self):
        """PDG codes of the beam and the two central particles of the process, followed for
        decay cascades by the four daughters."""
        from .modeldata import PARTICLES
        tree = _card.decay_tree(self.process.split("@")[0].split("->", 1)[1])
        out = [PARTICLES["p+"][0]] + [PARTICLES[name][0] for name, _ in tree]
        for _, kids in tree:
            out += [PARTICLES[name][0] for name, _ in kids]
        return out


def kernel_timing(engine, reset=True):
    """(total ms, launches) of the VEGAS sampling kernel since the last reset."""
    ms, n = ctypes.c_double(), ctypes.c_int64()
    _abi.check(engine.lib.grn_kernel_timing(engine.h, 1 if reset else 0, ctypes.byref(ms),
                                            ctypes.byref(n)))
    return ms.value, n.value


def fp32_peak(device=0):
    lib = _abi.load_library()
    t = ctypes.c_double()
    _abi.check(lib.grn_fp32_peak(device, ctypes.byref(t)))
    return t.value

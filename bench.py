"""Benchmark: unweighted events/s of the screened pi+ pi- continuum on one GB300.

Workload (the screened configuration of the generator):
  PP[CON]<C> -> pi+ pi-, sqrt(s) = 13 TeV, TUNE0, |eta| < 0.9, pT > 0.1 GeV,
  eikonal screening with a 1024-interval impact-parameter density table and a
  10000-interval kt^2 screening table, kt-loop of 63 x 33 intervals (64 x 34 points)
  with kt <= 3 GeV; 2^22 points per integration pass, VEGAS grid of 128 bins per
  dimension.
A step is one integration pass: points -> (flow) -> VEGAS map -> event weight (FP64
kinematics, FP32 compensated kt-loop) -> f = W vw / q -> sums and max.

Three samplers run on the same engine, in this order:
  plain VEGAS, mixed precision   burn-in, then timed passes (grid refined each pass)
  flow proposal (the headline)   one flow per seed (3 seeds), each trained (untimed,
                                 reported) in 4 rounds of 3 epochs, batch 16384, on 2^22
                                 weighted points each (round 1 from the adapted grid, later
                                 rounds from the flow itself), then timed passes, grid
                                 frozen; 5% of each pass is drawn uniformly (defensive
                                 mixture); the headline is the median seed, min and max
                                 are reported
  plain VEGAS, FP64 throughout   two timed passes on the adapted grid
value  = evaluations/s x eps_unw of the flow passes (median over the seeds),
         eps_unw = <f>/max f (reference semantics: max f over the integration passes),
         points generated on the device. Every reduction of a pass is in a fixed order
         (no floating-point atomics), so a run is reproducible bit for bit.
e2e    = unweighted events delivered to pinned host memory through the C ABI:
         grn_flow_iteration + grn_unweight (hit-or-miss against that max f) +
         grn_vegas_points, timed on the host clock.

Two more legs run the mixed workload of uneven multiplicity (screened tensor-pomeron
f2(1270) -> pi+ pi-, pi+ pi- continuum and rho rho -> pi+ pi- pi+ pi- with on-shell rho, all
in the continuum class, 50/30/20, on the same loop grid): at 2^24 points per pass on plain
VEGAS (batched against one member after another and against plain FP64), and its full form
at 2^26 points per pass with a learned proposal on every member (rho rho: 8 coupling layers
of width 256 over its 12 dimensions), batched, against plain VEGAS and plain FP64.

--impl reference times the CPU restatement of the reference path (oracle port, all
host threads) running plain VEGAS on the same workload, metric and unit.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

CARD_SCR = os.path.join(REPO, "tests", "golden", "cards", "pp_con_pipi_screened.json")
METRIC = "unweighted events/s at 0.1% sigma stat err (screened pi+pi- continuum, VEGAS)"
UNIT = "events/s"
N_BT, N_KT2, LOOP_KT, LOOP_PHI, LOOP_KTMAX = 1024, 10000, 63, 33, 3.0
LOOP_POINTS = (LOOP_KT + 1) * (LOOP_PHI + 1)
TRAFFIC_FILE = os.path.join(REPO, "profiles", "k_vegas_loop_rec_traffic.json")


def workload_params():
    from graniitti_gb300 import card
    P = card.build_params(card.read_card(CARD_SCR))
    P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = LOOP_KT, LOOP_PHI, LOOP_KTMAX
    P.loop.n_bt, P.loop.n_kt2 = N_BT, N_KT2
    return P


def config(n_points, world):
    return {"workload": "PP[CON]<C> -> pi+ pi- screened, 13 TeV TUNE0, VEGAS 128 bins x 8 dims",
            "points_per_step": n_points, "loop_points_per_event": LOOP_POINTS,
            "eikonal_tables": [N_BT, N_KT2], "loop_kt_max_gev": LOOP_KTMAX,
            "parallelism": "replicas x%d" % world,
            "l2_policy": "inputs larger than L2: 2^22 x 8 B f-array written per step; "
                         "points generated in-kernel"}


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in self.lines:
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def flops_per_loop_point():
    """FP32 operations per kt-loop point from the instrumented count of the
    product's loop arithmetic (graniitti_gb300/csrc/flopcount.cc)."""
    from graniitti_gb300 import flops
    return flops.loop_point_counts()


def cpu_vegas_sample(P, msa, n_events, nthreads, seed=4242):
    """Oracle weights of n_events VEGAS-uniform points (uniform grid)."""
    from oracle import oracle_api as orc
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import philox_np
    u = philox_np.uniforms(seed, n_events, 8)
    t0 = time.perf_counter()
    w, fl = orc.weights(P, u, msa=msa, nthreads=nthreads)
    return time.perf_counter() - t0, w


def run_reference(args, rank, world):
    """CPU arm: the oracle port of the reference path runs plain VEGAS on all host
    threads (grid adaptation with the oracle's map/refine), bounded samples."""
    if rank != 0:
        return
    from oracle import oracle_api as orc
    sys.path.insert(0, os.path.join(REPO, "tests"))
    import philox_np
    P = workload_params()
    nthreads = os.cpu_count() or 1
    mbt, msa, xs = orc.eikonal(P, N_BT, N_KT2, nthreads=nthreads)
    # size the per-step sample to ~2 s of CPU work
    dt, _ = cpu_vegas_sample(P, msa, 64 * nthreads, nthreads)
    rate = 64 * nthreads / dt
    n_step = int(max(1024, min(1 << 20, 2.0 * rate)))
    xmat = orc.vegas_grid_init(128, 8)

    def one_iter(it, track):
        u = philox_np.uniforms(77, n_step, 8, stream=it)
        x, vw, bins = orc.vegas_map(xmat, u)
        w, _ = orc.weights(P, x, msa=msa, nthreads=nthreads)
        f = w * vw
        f2 = np.zeros((128, 8))
        for j in range(8):
            np.add.at(f2[:, j], bins[:, j] - 1, f * f)
        return f, f2

    for it in range(args.warmup):
        f, f2 = one_iter(it, False)
        xmat = orc.vegas_refine(xmat, f2)
    fs, maxf = [], 0.0
    t0 = time.perf_counter()
    for it in range(args.steps):
        f, f2 = one_iter(1000 + it, True)
        xmat = orc.vegas_refine(xmat, f2)
        fs.append(f.mean())
        maxf = max(maxf, f.max())
    elapsed = time.perf_counter() - t0
    eps = float(np.mean(fs) / maxf) if maxf > 0 else 0.0
    value = n_step * args.steps * eps / elapsed
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * elapsed / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": dict(config(n_step, 1), eps_unw=eps, evaluations_per_s=n_step * args.steps /
                           elapsed),
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": "%d VEGAS-mapped points per step, %d timed steps, "
                                       "oracle port on %d host threads" %
                                       (n_step, args.steps, nthreads)},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


FLOW_LAYERS, FLOW_BATCH, FLOW_LR, FLOW_MIX = 6, 16384, 1e-3, 0.05
# multiply-adds of the conditioner per point and layer: 4x128, 128x128, 128x196
FLOW_FLOPS_PER_POINT = FLOW_LAYERS * 2 * (4 * 128 + 128 * 128 + 128 * 196)


def _timed_passes(torch, stream, fn, steps):
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    out = [fn(it) for it in range(steps)]
    t1.record(stream)
    torch.cuda.synchronize()
    return t0.elapsed_time(t1), out


def _summary(results, ms, npts, steps):
    """Unweighted events/s and the time to a 0.1% statistical error of a run."""
    r = results[-1]
    eps = r.sigma / r.maxf if r.maxf > 0 else 0.0
    evals_s = npts * steps / (ms * 1e-3)
    rel_var = max(r.I2_this * npts / r.I_this ** 2, 0.0) if r.I_this else None
    t01 = rel_var / 1e-6 / evals_s if rel_var is not None else None
    return {"value": evals_s * eps, "eps_unw": eps, "evaluations_per_s": evals_s,
            "sigma_barn": r.sigma, "sigma_rel_err": r.sigma_err / r.sigma if r.sigma else None,
            "rel_var_per_point": rel_var, "seconds_to_0.1pct": t01, "ms_per_step": ms / steps}


# The mixed workload of uneven multiplicity (continuum class <C>, screened, the 63 x 33 loop
# grid with kt <= 3 GeV of the screened pi+ pi- configuration): tensor-pomeron
# f2(1270) -> pi+ pi- (2-body, 8 dims), the tensor-pomeron pi+ pi- continuum (2-body, 8 dims)
# and tensor-pomeron rho rho -> pi+ pi- pi+ pi- with on-shell rho (4-body, 12 dims), 50/30/20;
# flow shapes per member for the full form.
RR_C = "PP[CONTENSOR]<C> -> rho(770)0 > {pi+ pi-} rho(770)0 > {pi+ pi-} @OFFSHELL:0"
MIX = [("PP[RESTENSOR]<C> -> pi+ pi- @RES{f2_1270:1}", 0.5, (6, 128)),
       ("PP[CONTENSOR]<C> -> pi+ pi-", 0.3, (6, 128)),
       (RR_C, 0.2, (8, 256))]
MIX_POINTS, FULL_POINTS, BURN_POINTS = 1 << 24, 1 << 26, 1 << 22


def _mix_workload(total, flows=False):
    s = ("screened tensor-pomeron f2(1270) -> pi+ pi- (<C>, 8 dims) + pi+ pi- continuum (<C>, 8 "
         "dims) + rho rho -> 4 pi (<C>, @OFFSHELL:0, 12 dims), %s of %d points per pass, loop "
         "grid %d x %d (kt <= %g GeV), one batched pass" %
         ("/".join(str(int(f * 100)) for _, f, _ in MIX), total, LOOP_KT, LOOP_PHI, LOOP_KTMAX))
    if flows:
        s += ", a learned proposal on every member (%s)" % ", ".join(
            "%d x %d" % sh for _, _, sh in MIX)
    return s


def mix_engines(g, _abi, total, burn, device, seed0):
    """The MIX members with their share of `total` points per pass, grids adapted by `burn`
    refined plain-VEGAS passes over BURN_POINTS points (untimed set-up)."""
    from graniitti_gb300 import card
    c = card.read_card(CARD_SCR)
    c["PROCESSPARAM"]["RES"] = ["f2_1270"]
    es = []
    for k, (proc, frac, _) in enumerate(MIX):
        P = card.build_params(c, proc)
        P.loop.n_kt, P.loop.n_phi, P.loop.kt_max = LOOP_KT, LOOP_PHI, LOOP_KTMAX
        P.loop.n_bt, P.loop.n_kt2 = N_BT, N_KT2
        e = g.Engine(P, device)
        e.eikonal_build(N_BT, N_KT2)
        vp = _abi.VegasParams()
        vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, 5, int(BURN_POINTS * frac) // 128 * 128, 1.5
        vp.chi2max, vp.precision, vp.burnin_iter = 10.0, 1e-3, burn
        vp.prec, vp.seed = g.MIXED, seed0 + k
        e.vegas_init(vp)
        for it in range(burn):
            e.vegas_iteration(mode=0, refine=True, iter_id=1 + it)
        grid = e.vegas_grid()
        vp.ncall = int(total * frac) // 128 * 128
        e.vegas_init(vp)
        e.vegas_set_grid(grid)
        e.vp = vp
        es.append(e)
    return es


def _timed_batch(torch, b, es, steps, refine, iter0):
    for e in es:
        e.vegas_clear()
        e.set_maxweight(0.0)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record()
    for it in range(steps):
        res, _ = b.iteration(mode=1, refine=refine, iter_id=iter0 + it)
    t1.record()
    torch.cuda.synchronize()
    return res, t0.elapsed_time(t1) / steps


def _fp64_pass_ms(g, _abi, torch, es, frac_points=64):
    """Plain FP64 VEGAS, member after member: the pass time at each member's full point count
    from a pass over 1/frac_points of its points on the same adapted grid."""
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    total = 0.0
    for e in es:
        grid, vp = e.vegas_grid(), e.vp
        vq = _abi.VegasParams()
        ctypes_copy(vq, vp)
        vq.ncall, vq.prec = max(128, int(vp.ncall) // frac_points // 128 * 128), g.FP64
        e.vegas_init(vq)
        e.vegas_set_grid(grid)
        torch.cuda.synchronize()
        t0.record()
        e.vegas_iteration(mode=1, refine=False, iter_id=900)
        t1.record()
        torch.cuda.synchronize()
        total += t0.elapsed_time(t1) * (int(vp.ncall) / int(vq.ncall))
        e.vegas_init(vp)
        e.vegas_set_grid(grid)
        e.vp = vp
    return total


def _member_stats(es, res, ms):
    out = []
    for (proc, frac, _), e, r in zip(MIX, es, res):
        n = int(e.vp.ncall)
        rel_var = max(r.I2_this * n / r.I_this ** 2, 0.0) if r.I_this else None
        evals_s = n / (ms * 1e-3)
        out.append({"process": proc, "points_per_step": n,
                    "eps_unw": r.sigma / r.maxf if r.maxf > 0 else None,
                    "sigma_barn": r.sigma, "sigma_rel_err": r.sigma_err / r.sigma if r.sigma else None,
                    "rel_var_per_point": rel_var, "refined_fp64": int(r.refined),
                    "seconds_to_0.1pct": rel_var / 1e-6 / evals_s if rel_var else None})
    return out


def mix_leg(g, _abi, torch, steps, burn, device):
    """The mixed workload at MIX_POINTS points per pass on plain VEGAS: one batched pass (fused
    stage A, graph-replayed) against the members one after another, and plain FP64."""
    es = mix_engines(g, _abi, MIX_POINTS, burn, device, 500)
    grids = [e.vegas_grid() for e in es]
    b = g.Batch(es)
    res_b, ms_b = _timed_batch(torch, b, es, steps, False, 100)
    b.close()
    for e, x in zip(es, grids):
        e.vegas_clear()
        e.set_maxweight(0.0)
        e.vegas_set_grid(x)
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    t0.record()
    for it in range(steps):
        res_s = [e.vegas_iteration(mode=1, refine=False, iter_id=100 + it) for e in es]
    t1.record()
    torch.cuda.synchronize()
    ms_s = t0.elapsed_time(t1) / steps
    ms64 = _fp64_pass_ms(g, _abi, torch, es)
    out = {"workload": _mix_workload(MIX_POINTS), "steps": steps,
           "ms_per_step_batched": ms_b, "ms_per_step_separate": ms_s,
           "ms_per_step_fp64_separate": ms64,
           "evaluations_per_s_batched": MIX_POINTS / (ms_b * 1e-3),
           "speedup_over_separate": ms_s / ms_b,
           "unweighted_per_s": {"plain_batched": _unweighted_per_s(es, res_b, ms_b),
                                "plain_separate": _unweighted_per_s(es, res_s, ms_s),
                                "plain_fp64_separate": _unweighted_per_s(es, res_s, ms64)},
           "processes": _member_stats(es, res_b, ms_b)}
    for e in es:
        e.close()
    return out


def full_form_leg(g, _abi, torch, steps, burn, device):
    """The full form at FULL_POINTS points per pass: every member draws its points from a
    learned proposal (rho rho: 8 coupling layers of width 256 over its 12 dimensions; the
    2-body members 6 of width 128), trained untimed in front of its adapted grid, all members
    in one batched pass; against the same members on plain VEGAS (batched) and on plain FP64
    VEGAS (member after member)."""
    es = mix_engines(g, _abi, FULL_POINTS, burn, device, 700)
    flows, trs = [], []
    for k, (e, (_, _, (layers, hidden))) in enumerate(zip(es, MIX)):
        f = g.Flow(e, layers=layers, hidden=hidden, seed=5 + k, mix_uniform=0.05)
        nt = max(16384, int(BURN_POINTS * MIX[k][1]) // 16384 * 16384)
        trs.append(f.train(n_train=nt, batch=16384, epochs=3, rounds=3, lr=1e-3, prec=g.MIXED,
                           seed_stream=7 + k))
        flows.append(f)
    grids = [e.vegas_grid() for e in es]
    bf = g.Batch(es)
    for k, f in enumerate(flows):
        bf.set_flow(k, f)
    res_f, ms_f = _timed_batch(torch, bf, es, steps, False, 300)
    bf.close()
    for e, x in zip(es, grids):
        e.vegas_set_grid(x)
    b = g.Batch(es)
    res_p, ms_p = _timed_batch(torch, b, es, steps, False, 400)
    b.close()
    ms64 = _fp64_pass_ms(g, _abi, torch, es)
    for f in flows:
        f.close()
    u_flow = _unweighted_per_s(es, res_f, ms_f)
    u_plain = _unweighted_per_s(es, res_p, ms_p)
    u_fp64 = _unweighted_per_s(es, res_p, ms64)
    out = {"workload": _mix_workload(FULL_POINTS, flows=True), "steps": steps,
           "flow": "RQ splines 16 bins, BF16 (tcgen05), 5% uniform mixture, trained untimed "
                   "(3 rounds x 3 epochs, batch 16384) on the adapted grids",
           "train_ms": [t.train_ms for t in trs], "train_steps": [t.steps for t in trs],
           "rel_var_train": {"plain": [t.rel_var_start for t in trs],
                             "flow": [t.rel_var_flow for t in trs]},
           "ms_per_step_flow_batched": ms_f, "ms_per_step_plain_batched": ms_p,
           "ms_per_step_fp64_separate": ms64,
           "unweighted_per_s": {"flow_batched": u_flow, "plain_batched": u_plain,
                                "plain_fp64_separate": u_fp64},
           "flow_batched_over_plain": u_flow / u_plain if u_plain else None,
           "flow_batched_over_plain_fp64": u_flow / u_fp64 if u_fp64 else None,
           "processes_flow": _member_stats(es, res_f, ms_f),
           "processes_plain": _member_stats(es, res_p, ms_p),
           "sigma_flow_vs_plain_pull": [
               (rf.sigma - rp.sigma) / (rf.sigma_err ** 2 + rp.sigma_err ** 2) ** 0.5
               for rf, rp in zip(res_f, res_p)]}
    for e in es:
        e.close()
    return out


def _unweighted_per_s(es, res, ms):
    """Unweighted events per second of a pass over all members: sum_p ncall_p eps_p / time,
    eps_p = <f>/max f of member p over its integration passes."""
    return sum(int(e.vp.ncall) * (r.sigma / r.maxf) for e, r in zip(es, res) if r.maxf > 0) / (
        ms * 1e-3)


def ctypes_copy(dst, src):
    import ctypes
    ctypes.memmove(ctypes.byref(dst), ctypes.byref(src), ctypes.sizeof(src))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--points", type=int, default=1 << 22)
    ap.add_argument("--flow-epochs", type=int, default=3)
    ap.add_argument("--flow-rounds", type=int, default=4)
    ap.add_argument("--flow-seeds", type=int, default=3)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-batch", action="store_true")
    ap.add_argument("--mix-steps", type=int, default=2,
                    help="timed passes of the mixed-workload legs (2^24 and 2^26 points)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")

    if args.impl == "reference":
        run_reference(args, rank, world)
        if dist:
            dist.barrier()
        return

    import ctypes

    import torch
    import graniitti_gb300 as g
    from graniitti_gb300 import _abi
    from graniitti_gb300.engine import fp32_peak, kernel_timing

    torch.cuda.set_device(local)
    P = workload_params()
    eng = g.Engine(P, local)
    eng.eikonal_build(N_BT, N_KT2)
    vp = _abi.VegasParams()
    vp.bins, vp.iter, vp.ncall, vp.lambda_ = 128, args.steps, args.points, 1.5
    vp.chi2max, vp.precision, vp.burnin_iter = 10.0, 1e-3, args.warmup
    vp.prec, vp.seed = g.MIXED, 1000 + rank
    eng.vegas_init(vp)
    stream = torch.cuda.ExternalStream(eng.stream)
    n = args.points

    # -- plain VEGAS, mixed precision: burn-in, then timed integration passes ----
    for it in range(args.warmup):
        eng.vegas_iteration(mode=0, refine=True, iter_id=1 + it)
    # the engine's autotuner picks the kt-loop kernel variant and grid on the loop stage of a
    # full pass over the adapted grid (untimed set-up)
    tune = eng.autotune()
    variant = {0: "1 event/thread", 1: "2 events/thread", 2: "2 events/thread, 3 blocks/SM"}

    def _label(k):
        c = tune.cand[k]
        if tune.stage[k] == 0:
            return "stage A x %d blocks" % c.born_blocks
        if tune.stage[k] == 2:
            return "generic loop x %d blocks" % c.generic_blocks
        return "%s x %d blocks" % (variant[c.loop_pair], c.vegas_blocks)
    tuned = {"loop_variant": variant[tune.best.loop_pair],
             "loop_blocks": tune.best.vegas_blocks,
             "stage_a_blocks": tune.best.born_blocks,
             "candidates_ms": {_label(k): round(tune.ms[k], 4) for k in range(tune.n_candidates)},
             "listed_events": tune.sample_events}
    eng.vegas_clear()
    ms_plain, res_plain = _timed_passes(
        torch, stream, lambda it: eng.vegas_iteration(mode=1, refine=True, iter_id=100 + it),
        args.steps)
    plain = _summary(res_plain, ms_plain, n, args.steps)
    xmat = eng.vegas_grid()

    # -- flow proposal in front of the adapted grid (training untimed, reported) -
    #    one flow per seed; the headline is the median over the seeds (eps_unw is a
    #    maximum-weight statistic and moves with the trained density's extreme tail)
    clocks = ClockSampler(local)
    clocks.start()
    runs = []
    k_ms, k_n = 0.0, 0
    for k in range(args.flow_seeds):
        flow = g.Flow(eng, layers=FLOW_LAYERS, seed=1 + k + 100 * rank, mix_uniform=FLOW_MIX)
        tr = flow.train(n_train=n, batch=FLOW_BATCH, epochs=args.flow_epochs,
                        rounds=args.flow_rounds, lr=FLOW_LR, prec=g.MIXED, seed_stream=1 + k)
        eng.vegas_clear()
        for it in range(2):
            flow.iteration(mode=0, iter_id=200 + it)
        eng.vegas_clear()
        eng.set_maxweight(0.0)  # the flow integration keeps its own maximum weight
        kernel_timing(eng, reset=True)
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        ms_k, res_k = _timed_passes(torch, stream,
                                    lambda it: flow.iteration(mode=1, iter_id=300 + it),
                                    args.steps)
        km, kn = kernel_timing(eng, reset=True)
        k_ms, k_n = k_ms + km, k_n + kn
        if dist:
            t = torch.tensor([ms_k], dtype=torch.float64)
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms_k = float(t[0])
        fl_k = _summary(res_k, ms_k, n, args.steps)
        runs.append({"flow": flow, "tr": tr, "ms": ms_k, "res": res_k, "fl": fl_k,
                     "value": n * args.steps * world * fl_k["eps_unw"] / (ms_k * 1e-3)})
    clk = clocks.stop()
    order = sorted(range(len(runs)), key=lambda k: runs[k]["value"])
    med = runs[order[len(order) // 2]]
    for k in order:
        if runs[k] is not med:
            runs[k]["flow"].close()
    flow, tr, ms, res_flow, fl = med["flow"], med["tr"], med["ms"], med["res"], med["fl"]
    r = res_flow[-1]
    fl_maxf = r.maxf
    eps = fl["eps_unw"]
    evals = n * args.steps * world
    value = med["value"]
    per_seed = [{"seed": 1 + k, "value": rk["value"], "eps_unw": rk["fl"]["eps_unw"],
                 "ms_per_step": rk["ms"] / args.steps, "sigma_barn": rk["fl"]["sigma_barn"],
                 "rel_var_per_point": rk["fl"]["rel_var_per_point"],
                 "train_ms": rk["tr"].train_ms} for k, rk in enumerate(runs)]

    # -- flow kernel alone (sampling direction, device buffers, engine stream) ---
    xs_dev = torch.empty((8, n), dtype=torch.float32, device="cuda")
    lq_dev = torch.empty(n, dtype=torch.float32, device="cuda")
    def _sample(it):
        _abi.check(eng.lib.grn_flow_sample(flow.h, 99, 500 + it, 0, n,
                                           ctypes.c_void_p(xs_dev.data_ptr()),
                                           ctypes.c_void_p(lq_dev.data_ptr())))
    _sample(0)
    ms_f, _ = _timed_passes(torch, stream, _sample, 3)
    flow_s = ms_f / 3 * 1e-3
    flow_tflops = n * FLOW_FLOPS_PER_POINT / flow_s / 1e12
    bf16_peak = None
    peaks_file = os.path.join(REPO, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_file):
        bf16_peak = json.load(open(peaks_file)).get("bf16_tflops")

    # -- plain VEGAS, FP64 throughout, on the same adapted grid ----------------
    fp64 = None
    if not args.no_fp64:
        vp64 = _abi.VegasParams.from_buffer_copy(vp)
        vp64.prec = g.FP64
        eng.vegas_init(vp64)
        eng.vegas_set_grid(xmat)
        eng.vegas_iteration(mode=0, refine=True, iter_id=400)
        eng.vegas_clear()
        eng.set_maxweight(0.0)
        k64 = 2
        ms64, res64 = _timed_passes(
            torch, stream, lambda it: eng.vegas_iteration(mode=1, refine=True, iter_id=410 + it),
            k64)
        fp64 = _summary(res64, ms64, n, k64)
        eng.vegas_init(vp)
        eng.vegas_set_grid(xmat)
        eng.set_maxweight(fl_maxf)
        kernel_timing(eng, reset=True)

    # -- several processes in one pass (fused launches, CUDA graph): the mixed workload
    #    on plain VEGAS, and its full form with a learned proposal on every member --------
    mixed = None if args.no_batch else mix_leg(g, _abi, torch, args.mix_steps, 3, local)
    full = None if args.no_batch else full_form_leg(g, _abi, torch, args.mix_steps, 3, local)

    # -- e2e: unweighted events delivered to pinned host memory through the C ABI
    #    (flow pass -> hit-or-miss against the integration's max f -> points) ---
    fmax = r.maxf
    idx_h = torch.empty(n, dtype=torch.int64).pin_memory()
    pts_h = torch.empty((n, 8), dtype=torch.float64).pin_memory()
    na, no = ctypes.c_int64(), ctypes.c_int64()

    def gen_step(it):
        flow.iteration(mode=2, iter_id=600 + it)
        _abi.check(eng.lib.grn_unweight(eng.h, fmax, 17 + it, ctypes.byref(na), ctypes.byref(no),
                                        ctypes.c_void_p(idx_h.data_ptr()), n))
        _abi.check(eng.lib.grn_vegas_points(eng.h, ctypes.c_void_p(idx_h.data_ptr()), na.value,
                                            ctypes.c_void_p(pts_h.data_ptr())))
        return na.value

    gen_step(0)
    torch.cuda.synchronize()
    e2e_steps = args.steps
    t0 = time.perf_counter()
    accepted = [gen_step(1 + it) for it in range(e2e_steps)]
    e2e_s = time.perf_counter() - t0
    e2e_value = sum(accepted) * world / e2e_s
    acc_step = sum(accepted) / e2e_steps

    # -- roofline of the dominant kernel (kt-loop stage of a pass) -------------
    cnt = flops_per_loop_point()
    passed = r.fidcuts_ok / r.evaluations if r.evaluations else 0.0
    flops_launch = n * passed * LOOP_POINTS * cnt["flops"]
    k_avg_s = (k_ms / max(k_n, 1)) * 1e-3
    peak = fp32_peak(local)
    achieved = flops_launch / k_avg_s / 1e12
    traffic = None
    if os.path.exists(TRAFFIC_FILE):
        traffic = json.load(open(TRAFFIC_FILE)).get("bytes_per_launch")

    cfg = dict(config(n, world), sigma_barn=r.sigma, sigma_rel_err=fl["sigma_rel_err"],
               eps_unw=eps, evaluations_per_s=evals / (ms * 1e-3), fid_pass=passed,
               sampler="flow proposal (6 coupling layers, RQ splines 16 bins, MLP 128x2, "
                       "BF16/FP32; 5%% uniform defensive component) in front of the adapted "
                       "VEGAS grid; FP64 kinematics, FP32 compensated kt-loop",
               value_median_of_seeds=len(runs),
               value_min=min(rk["value"] for rk in runs),
               value_max=max(rk["value"] for rk in runs),
               flow_seeds=per_seed,
               flow=dict(fl, train_ms=tr.train_ms, train_steps=tr.steps, batch=FLOW_BATCH,
                         epochs=args.flow_epochs, rounds=args.flow_rounds, mix_uniform=FLOW_MIX,
                         rel_var_vegas_points=tr.rel_var_start,
                         rel_var_flow_points=tr.rel_var_flow,
                         sample_kernel_ms=flow_s * 1e3, sample_tflops=flow_tflops,
                         sample_frac_of_measured_bf16=(flow_tflops / bf16_peak
                                                       if bf16_peak else None)),
               plain_vegas_mixed=plain, plain_vegas_fp64=fp64, autotune=tuned,
               mixed_workload=mixed, full_form=full,
               flow_over_plain_mixed=value / plain["value"] if plain["value"] else None,
               flow_over_plain_fp64=(value / fp64["value"]) if fp64 and fp64["value"] else None)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32+bf16", "data": "synthetic",
            "config": cfg,
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(acc_step * 8),
                    "d2h_bytes_per_step": int(acc_step * (8 + 64) + 2 * 8 + 8 * 10),
                    "what": "grn_flow_iteration + grn_unweight + grn_vegas_points per step, "
                            "accepted events' hypercube vectors into pinned host memory"},
            # per flow pass: uniform points, density of the uniform share, flow sample,
            # mixture density (4), stage A, kt-loop stage, sums, finish (4)
            "gpu_launches": (8 if FLOW_MIX > 0 else 5) * args.steps,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                         "traffic": traffic,
                         "peak_source": "measured FP32 FMA-chain probe (MEASURED_PEAKS.json "
                                        "carries no FP32 figure)",
                         "kernel": {0: "k_vegas_loop_rec",
                                    1: "k_vegas_loop_rec2<2> (2 events per thread, packed FP32x2)",
                                    2: "k_vegas_loop_rec2<3> (2 events per thread, packed FP32x2, "
                                       "3 blocks per SM)"}[tune.best.loop_pair],
                         "flops_per_loop_point": cnt["flops"],
                         "sfu_per_loop_point": cnt["transcendentals"],
                         "kernel_ms": k_avg_s * 1e3},
            "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        nthreads = os.cpu_count() or 1
        _, msa = eng.eikonal_tables(N_BT, N_KT2)
        n_cpu = 16 * nthreads
        dt, _ = cpu_vegas_sample(P, msa, n_cpu, nthreads)
        n_cpu = int(min(1 << 18, max(n_cpu, n_cpu * 10.0 / max(dt, 1e-3))))
        dt, _ = cpu_vegas_sample(P, msa, n_cpu, nthreads, seed=4343)
        line["cpu_baseline"] = {"value": n_cpu / dt * plain["eps_unw"], "unit": UNIT,
                                "cores": nthreads, "kind": "port",
                                "sample": "%d uniform points of the same workload through the "
                                          "oracle port on %d threads (%.1f s), x the plain-VEGAS "
                                          "eps_unw of the GPU run" % (n_cpu, nthreads, dt)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    flow.close()
    eng.close()
    if dist:
        dist.barrier()


if __name__ == "__main__":
    main()

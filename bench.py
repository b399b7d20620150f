"""Benchmark: unweighted events/s of the screened pi+ pi- continuum on one GB300.

Workload (the screened configuration of the generator):
  PP[CON]<C> -> pi+ pi-, sqrt(s) = 13 TeV, TUNE0, |eta| < 0.9, pT > 0.1 GeV,
  eikonal screening with a 1024-interval impact-parameter density table and a
  10000-interval kt^2 screening table, kt-loop of 63 x 33 intervals (64 x 34 points)
  with kt <= 3 GeV; 2^22 Philox points per VEGAS iteration, 128 bins per dimension.
A step is one VEGAS iteration: points -> grid map -> event weight (FP64 kinematics,
FP32 compensated kt-loop) -> f, f^2 histograms -> grid refinement.

value  = evaluations/s x eps_unw over the timed iterations, eps_unw = <f>/max f
         (reference semantics: max f over integration iterations), inputs resident
         on the device (counter-based points generated in the kernel).
e2e    = the same metric through grn_event_weights with pinned HOST buffers: the
         VEGAS-mapped points of a step are copied in and the weights out inside
         the timed region.

--impl reference times the CPU restatement of the reference path (oracle port, all
host threads) on the same workload, metric and unit.
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
TRAFFIC_FILE = os.path.join(REPO, "profiles", "vegas_sample_c2_traffic.json")  # k_vegas_loop


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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine", choices=["engine", "reference"])
    ap.add_argument("--points", type=int, default=1 << 22)
    ap.add_argument("--no-cpu-baseline", action="store_true")
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
    # burn-in (untimed): grid adaptation
    for it in range(args.warmup):
        eng.vegas_iteration(mode=0, refine=True, iter_id=1 + it)
    eng.vegas_clear()
    kernel_timing(eng, reset=True)
    stream = torch.cuda.ExternalStream(eng.stream)

    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    time.sleep(0.3)
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    results = []
    for it in range(args.steps):
        results.append(eng.vegas_iteration(mode=1, refine=True, iter_id=100 + it))
    t_end.record(stream)
    torch.cuda.synchronize()
    clk = clocks.stop()
    ms = t_start.elapsed_time(t_end)
    k_ms, k_n = kernel_timing(eng, reset=True)
    if dist:
        t = torch.tensor([ms], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t[0])
    r = results[-1]
    eps = r.sigma / r.maxf if r.maxf > 0 else 0.0
    evals = args.points * args.steps * world
    value = evals * eps / (ms * 1e-3)

    # -- e2e through the C ABI with pinned host buffers ------------------------
    idx = np.arange(args.points, dtype=np.int64)
    x_host = torch.empty((args.points, 8), dtype=torch.float64).pin_memory()
    x_host.numpy()[:] = eng.vegas_points(idx)
    w_host = torch.empty(args.points, dtype=torch.float64).pin_memory()
    f_host = torch.empty(args.points, dtype=torch.uint8).pin_memory()
    xn, wn, fn = x_host.numpy(), w_host.numpy(), f_host.numpy()
    eng.event_weights(xn, prec=g.MIXED, w=wn, flags=fn)  # warm
    torch.cuda.synchronize()
    e2e_steps = max(2, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        eng.event_weights(xn, prec=g.MIXED, w=wn, flags=fn)
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    e2e_value = args.points * world * eps / e2e_s

    # -- roofline of the dominant kernel (VEGAS sampling pass) -----------------
    cnt = flops_per_loop_point()
    passed = r.fidcuts_ok / r.evaluations if r.evaluations else 0.0
    # algorithmic work of one k_vegas_loop launch: listed (passing) events x loop points
    flops_launch = args.points * passed * LOOP_POINTS * cnt["flops"]
    k_avg_s = (k_ms / max(k_n, 1)) * 1e-3
    peak = fp32_peak(local)
    achieved = flops_launch / k_avg_s / 1e12
    traffic = None
    if os.path.exists(TRAFFIC_FILE):
        traffic = json.load(open(TRAFFIC_FILE)).get("bytes_per_launch")

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic",
            "config": dict(config(args.points, world), eps_unw=eps, sigma_barn=r.sigma,
                           sigma_rel_err=r.sigma_err / r.sigma if r.sigma else None,
                           evaluations_per_s=evals / (ms * 1e-3), fid_pass=passed),
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(args.points * 8 * 8),
                    "d2h_bytes_per_step": int(args.points * 9)},
            "gpu_launches": 5 * args.steps,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak,
                         "unit": "TFLOP/s", "frac": achieved / peak if peak else None,
                         "traffic": traffic,
                         "peak_source": "measured FP32 FMA-chain probe (MEASURED_PEAKS.json "
                                        "carries no FP32 figure)",
                         "flops_per_loop_point": cnt["flops"],
                         "sfu_per_loop_point": cnt["transcendentals"],
                         "kernel_ms": k_avg_s * 1e3},
            "clocks": clk}
    if rank == 0 and not args.no_cpu_baseline:
        from oracle import oracle_api as orc
        nthreads = os.cpu_count() or 1
        _, msa = eng.eikonal_tables(N_BT, N_KT2)
        n_cpu = 16 * nthreads
        dt, _ = cpu_vegas_sample(P, msa, n_cpu, nthreads)
        n_cpu = int(min(1 << 18, max(n_cpu, n_cpu * 10.0 / max(dt, 1e-3))))
        dt, _ = cpu_vegas_sample(P, msa, n_cpu, nthreads, seed=4343)
        line["cpu_baseline"] = {"value": n_cpu / dt * eps, "unit": UNIT, "cores": nthreads,
                                "kind": "port",
                                "sample": "%d uniform points of the same workload through the "
                                          "oracle port on %d threads (%.1f s), x the GPU run's "
                                          "eps_unw" % (n_cpu, nthreads, dt)}
    if rank == 0:
        print(json.dumps(line), flush=True)
    eng.close()
    if dist:
        dist.barrier()


if __name__ == "__main__":
    main()

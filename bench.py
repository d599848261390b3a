#!/usr/bin/env python
"""Benchmark: Levenberg-Marquardt bundle adjustment on one GB300 (or N replicas).

Workload (default): one large problem -- 88 cameras on a 200 m circle,
64,298 points, about 385k observations with power-law views per point (mean
about 6), 6-parameter cameras, fixed K, pixel noise N(0,1), 2% outliers --
solved by plain FP64 Levenberg-Marquardt for up to 50 iterations (the
LM->TR hand-over disabled).  A step is one full solve from the same initial
estimate.  The metric is LM iterations per second.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

* value: iterations / device time of the K solves with the problem resident
  in HBM (CUDA events on the solver's stream, bracketing each solve; the L2
  is flushed between solves and the per-iteration working set is larger
  than L2 anyway).
* e2e: the same metric through the C ABI from host buffers: psba_create
  (upload, index lists) + psba_levmar + psba_get_params per step, host clock.
* roofline: the dominant kernel, k_schur (the Schur complement's
  off-diagonal blocks in equal chunks of the pair list, and its diagonal
  blocks in the same launch; one launch per LM trial), timed live with CUDA
  events inside the timed solves; FP64-bound, so its peak is the measured
  FP64 FMA rate.
  roofline_chol: the same for the dense solve (k_chol_dataflow +
  k_tri_cluster).  Only these two stages carry events in the timed solves.
* stage_ms / stage_share and roofline_schur (the whole Schur-complement
  stage): from one more solve after the timed region with every stage timed
  (events around every stage cost ~4 us each on the stream).
* variable_intrinsics: 52 cameras x 64,053 points with 11- and
  16-parameter cameras, mixed and FP64 forms, LM iterations/s.
* batched: 1,024 small problems in one persistent launch (mixed form,
  autotuned shape) against the plain FP64 single-problem solver.
* serving: Poisson arrivals into the continuous-batching server (batch lane
  plus large lane), solves/s, p50/p99 latency per arrival rate.
* cpu_baseline: the FP64 CPU oracle (a C restatement of the reference's
  path) on the host cores, on a bounded sample of the same problem.
* --impl reference: the CPU oracle alone (the reference's OpenCL/MSVC path
  does not build on this machine), one LM iteration per step.
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

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "LM iterations/s (plain FP64 Levenberg-Marquardt, 88 cams x 64,298 pts)"
UNIT = "iterations/s"

# DRAM bytes (read + write) per launch from one ncu capture of this workload
# (profiles/k_schur_circle88.md, profiles/k_chol_dataflow_circle88.md).
SCHUR_TRAFFIC = 250.1e6
CHOL_TRAFFIC = 1.30e6  # profiles/k_chol_dataflow_circle88.md: S (2.2 MB) stays in L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--points", type=int, default=64298)
    ap.add_argument("--cams", type=int, default=88)
    ap.add_argument("--max-iter", type=int, default=50)
    ap.add_argument("--cpu-iters", type=int, default=2, help="oracle LM iterations in the CPU sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-form leg")
    ap.add_argument("--tr-iters", type=int, default=50, help="trust-region leg iterations (0: skip)")
    ap.add_argument("--varcam-iters", type=int, default=30, help="LM iterations of the variable-intrinsics leg (0: skip)")
    ap.add_argument("--batch", type=int, default=1024, help="problems in the batched leg (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--pbp-sample", type=int, default=64,
                    help="problems solved one by one by the plain FP64 form for the batched comparison")
    ap.add_argument("--serve-rates", default="50,200,1000,2000", help="Poisson rates, req/s ('none' to skip)")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="arrival window per rate")
    ap.add_argument("--serve-max", type=int, default=400, help="requests per rate at most")
    ap.add_argument("--serve-pool", type=int, default=32, help="distinct request scenes (cycled)")
    ap.add_argument("--serve-large-lanes", type=int, default=None, help="server large_lanes (default: library's)")
    ap.add_argument("--serve-large-obs", type=int, default=None, help="server large_obs (default: library's)")
    return ap.parse_args()


def workload_config(args, sc):
    k = np.bincount(sc.obs_pt)
    return {
        "workload": "LM bundle adjustment, %d cameras x %d points, %d observations (power-law views, mean %.2f), "
                    "6-param cameras, fixed K, %d iterations max, LM->TR switch off" % (
                        sc.n_cams, sc.n_pts, sc.n_obs, k.mean(), args.max_iter),
        "cameras": sc.n_cams, "points": sc.n_pts, "observations": sc.n_obs,
        "pair_entries": int(((k * (k - 1)) // 2).sum()),
        "max_iter": args.max_iter, "precision": "fp64",
        "l2": "flushed between solves (256 MiB write); per-iteration working set > L2",
    }


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.t.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs"), "measured"
    return 6800.0, "fallback"


def schur_bytes(sc):
    """Algorithmic bytes of the Schur stage per trial: Y and W of every
    observation (FP64), a 4-byte index per observation, and S (6C)^2 FP64."""
    O, C = sc.n_obs, sc.n_cams
    return 2 * O * 18 * 8 + O * 4 + (6 * C) ** 2 * 8


def schur_flops(cfg):
    """FP64 flops of the Schur stage per trial: 6x6x3 FMAs per off-diagonal
    pair entry, (21 + 6) x 3 FMAs per observation for the diagonal blocks and ea."""
    return 2 * 108 * cfg["pair_entries"] + 2 * 81 * cfg["observations"]


def flush_l2(torch, buf):
    buf.zero_()
    torch.cuda.synchronize()


def cpu_baseline(sc, args):
    import oracle
    nthreads = os.cpu_count() or 1
    sess = oracle.Session(sc)
    out = {}
    for tag, th in (("threads", nthreads), ("single", 1)):
        iters = args.cpu_iters if tag == "threads" else 1
        o = oracle.default_opts(allow_switch=0, max_iter=iters, n_threads=th)
        t = time.perf_counter()
        r = sess.levmar(o)
        dt = time.perf_counter() - t
        out[tag] = (r.iterations / dt, r, dt)
    sess.close()
    return out, nthreads


def run_reference(args):
    """The reference arm: the FP64 CPU restatement on all host cores, one LM
    iteration of the same problem per step (restarted from the initial
    estimate each step)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle
    from psba_gb300 import scenes
    sc = scenes.circle_scene(seed=0, n_cams=args.cams, n_pts=args.points, name="circle")
    cfg = workload_config(args, sc)
    nthreads = os.cpu_count() or 1
    sess = oracle.Session(sc)
    o = oracle.default_opts(allow_switch=0, max_iter=1, n_threads=nthreads)
    for _ in range(args.warmup):
        sess.levmar(o)
    t = time.perf_counter()
    iters = 0
    for _ in range(args.steps):
        iters += sess.levmar(o).iterations
    dt = time.perf_counter() - t
    sess.close()
    value = iters / dt
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": cfg, "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": "1 LM iteration of the same problem per step, %d steps" % args.steps},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def aggregate_replicas(torch, dist, dev_s, wall_s, iters, device):
    """Replicas only (no data-path collective): each rank solves its own
    problem; the job's time is the slowest rank's (device and wall clock),
    its work the sum of the ranks' iterations.  Returns (device seconds, wall
    seconds, iterations) for the whole job; single-process runs pass through."""
    if not dist:
        return dev_s, wall_s, iters
    t = torch.tensor([dev_s, wall_s], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    it = torch.tensor([float(iters)], dtype=torch.float64, device=device)
    dist.all_reduce(it, op=dist.ReduceOp.SUM)
    return float(t[0]), float(t[1]), float(it[0])


def batched_leg(P, args):
    """1,024 independent problems (5-30 cameras, 200-3,000 points, 3-8 views)
    in one persistent launch under a CUDA graph, 15 LM iterations each: the
    mixed form with the autotuned shape, the FP64 form in the same launch
    shape, and the plain FP64 single-problem solver one problem at a time on
    a sample of the same problems."""
    from psba_gb300 import batch as B
    from psba_gb300 import scenes
    probs = scenes.batch_scenes(args.batch, seed=1000)
    iters = 15
    mo = P.default_opts(allow_switch=0, max_iter=iters, precision=P.PREC_MIXED)
    fo = P.default_opts(allow_switch=0, max_iter=iters)
    with B.Batch(probs) as b:
        choice, table = B.autotune(b, P.PREC_MIXED, iters=1, repeats=1)
        b.reset()
        b.levmar(mo)
        m_ms = []
        for _ in range(args.batch_steps):
            b.reset()
            res_m, ms = b.levmar(mo)
            m_ms.append(ms)
        b.reset()
        b.levmar(fo)
        f_ms = []
        for _ in range(args.batch_steps):
            b.reset()
            res_f, ms = b.levmar(fo)
            f_ms.append(ms)
        dev_bytes = b.device_bytes()
    # the plain FP64 form, problem by problem (create outside the timing)
    sample = probs[: args.pbp_sample]
    pbp_ms, pbp_cost = [], []
    for sc in sample:
        with P.Solver(sc) as s:
            r = s.levmar(fo, fetch=False, trace_cap=0)
        pbp_ms.append(r.device_ms)
        pbp_cost.append(r.final_cost)
    rel = np.abs(res_m["final_cost"] - res_f["final_cost"]) / res_f["final_cost"]
    pbp_rel = np.abs(res_f["final_cost"][: len(sample)] - np.array(pbp_cost)) / np.array(pbp_cost)
    m_sps = args.batch / (min(m_ms) / 1e3)
    f_sps = args.batch / (min(f_ms) / 1e3)
    pbp_sps = len(sample) / (sum(pbp_ms) / 1e3)
    return {
        "workload": "%d problems, 5-30 cameras, 200-3,000 points, 3-8 views per point, %d LM iterations each, "
                    "one persistent launch under a CUDA graph" % (args.batch, iters),
        "observations": int(sum(sc.n_obs for sc in probs)), "device_bytes": int(dev_bytes),
        "mixed_solves_per_s": m_sps, "mixed_ms": min(m_ms),
        "fp64_batched_solves_per_s": f_sps, "fp64_batched_ms": min(f_ms),
        "fp64_problem_by_problem_solves_per_s": pbp_sps,
        "fp64_problem_by_problem_sample": len(sample),
        "speedup_mixed_batched_vs_fp64_problem_by_problem": m_sps / pbp_sps,
        "mixed_final_cost_rel_vs_fp64": {"max": float(rel.max()), "median": float(np.median(rel)),
                                          "frac_within_1e-6": float((rel <= 1e-6).mean())},
        "fp64_batched_vs_single_max_rel": float(pbp_rel.max()),
        "autotune": choice, "autotune_candidates": len(table),
    }


def varcam_leg(P, args):
    """Variable intrinsics: 52 cameras x 64,053 points (power-law views,
    mean 5.42), 11- and 16-parameter cameras, intrinsics 5% off, LM for
    --varcam-iters iterations in the mixed and the FP64 form."""
    from psba_gb300 import scenes
    out = {}
    for cnp in (11, 16):
        sc = scenes.varcam_scene(cnp, seed=0)
        res = {"cameras": sc.n_cams, "points": sc.n_pts, "observations": sc.n_obs, "N": cnp * sc.n_cams}
        with P.Solver(sc) as s:
            for tag, prec in (("mixed", P.PREC_MIXED), ("fp64", P.PREC_FP64)):
                o = P.default_opts(allow_switch=0, max_iter=args.varcam_iters, precision=prec)
                s.reset_params()
                s.levmar(o, fetch=False, trace_cap=0)  # warm-up
                s.reset_params()
                r = s.levmar(o, fetch=False, trace_cap=0)
                res[tag] = {"iterations_per_s": r.iterations / (r.device_ms / 1e3), "ms_per_solve": r.device_ms,
                            "iterations": r.iterations, "trials": r.n_trials, "initial_cost": r.initial_cost,
                            "final_cost": r.final_cost}
        res["mixed_final_cost_rel_vs_fp64"] = abs(res["mixed"]["final_cost"] - res["fp64"]["final_cost"]) / \
            res["fp64"]["final_cost"]
        res["speedup_mixed_vs_fp64"] = res["mixed"]["iterations_per_s"] / res["fp64"]["iterations_per_s"]
        out["cnp%d" % cnp] = res
    return out


def serving_leg(P, args):
    """Poisson arrivals of requests (cameras log-uniform 5-138, points
    500-60,000, 4-6 views, 6- or 11-parameter cameras) into the serving engine
    (mixed form, 15 LM iterations, 120 GB HBM budget); p50/p99 latency from
    submission to result on the host clock."""
    from psba_gb300 import scenes
    from psba_gb300 import serve as S
    rates = [float(x) for x in args.serve_rates.split(",") if x.strip()]
    pool = scenes.serving_scenes(args.serve_pool, seed=2000)
    # every other request scene with 11-parameter cameras (intrinsics 1% off)
    pool = [scenes.with_intrinsics(sc, 11, seed=3000 + q, k_off=0.01) if q % 2 else sc
            for q, sc in enumerate(pool)]
    iters = 15
    out = {"workload": "Poisson arrivals; %d distinct request scenes cycled: cameras log-U[5,138], points "
                       "log-U[500,60000], 4-6 views/point, half 6-param and half 11-param cameras, mixed form, "
                       "%d LM iterations, 120 GB HBM budget" % (len(pool), iters),
           "mean_observations": float(np.mean([sc.n_obs for sc in pool])), "rates": []}
    with S.Server(precision=P.PREC_MIXED, max_iter=iters, hbm_budget_bytes=120e9,
                  large_lanes=args.serve_large_lanes, large_obs=args.serve_large_obs) as srv:
        S.run_poisson(srv, pool[:4], rate=1000.0, n_requests=4, seed=1)
        first = {}
        for rate in rates:
            n = int(min(max(rate * args.serve_seconds, 20), args.serve_max))
            got, wall = S.run_poisson(srv, pool, rate, n, seed=int(rate))
            lat = np.array([r.latency_ms for r in got])
            qd = np.array([r.queued_ms for r in got])
            for q, r in enumerate(got):
                first.setdefault(q % len(pool), r.final_cost)
            out["rates"].append({"rate_req_s": rate, "requests": n, "solves_per_s": n / wall,
                                 "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                                 "queued_p50_ms": float(np.percentile(qd, 50)),
                                 "queued_p99_ms": float(np.percentile(qd, 99))})
        st = srv.stats()
    out["launches"] = st["launches"]
    out["peak_bytes"] = st["peak_bytes"]
    # final cost against the plain FP64 single-problem solver on the same scenes
    rel = []
    fo = P.default_opts(allow_switch=0, max_iter=iters)
    for q, c in sorted(first.items()):
        with P.Solver(pool[q]) as s:
            r = s.levmar(fo, fetch=False, trace_cap=0)
        rel.append(abs(c - r.final_cost) / r.final_cost)
    rel = np.array(rel)
    out["final_cost_rel_vs_fp64"] = {"max": float(rel.max()), "median": float(np.median(rel)),
                                     "frac_within_1e-6": float((rel <= 1e-6).mean())}
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    import psba_gb300 as P
    from psba_gb300 import scenes

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    P.lib()
    sc = scenes.circle_scene(seed=rank, n_cams=args.cams, n_pts=args.points, name="circle")
    cfg = workload_config(args, sc)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    opts = P.default_opts(allow_switch=0, max_iter=args.max_iter)

    solver = P.Solver(sc)
    for _ in range(args.warmup):
        solver.reset_params()
        solver.levmar(opts, fetch=False, trace_cap=0)

    # ---- timed region: K solves from the same initial estimate, problem resident in HBM.
    # Only the two roofline stages carry events here (each timed stage costs
    # two events per occurrence on the stream); the per-stage breakdown comes
    # from one more solve with every stage timed, after the timed region.
    solver.set_stage_timing(True, stages=("schur_off", "cholesky"))
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = P.kernel_launches()
    barrier()
    t0 = time.perf_counter()
    dev_ms, iters, trials, costs = [], 0, 0, []
    for _ in range(args.steps):
        solver.reset_params()
        flush_l2(torch, flush)
        r = solver.levmar(opts, fetch=False, trace_cap=0)
        dev_ms.append(r.device_ms)
        iters += r.iterations
        trials += r.n_trials
        costs.append(r.final_cost)
    barrier()
    wall = time.perf_counter() - t0
    launches = P.kernel_launches() - launches0
    clk = clocks.stop()
    live = solver.stage_timing()
    solver.set_stage_timing(True)
    solver.reset_params()
    solver.levmar(opts, fetch=False, trace_cap=0)
    stages = solver.stage_timing()
    solver.set_stage_timing(False)

    total_dev_s, wall, iters_all = aggregate_replicas(torch, dist, sum(dev_ms) / 1e3, wall, iters, "cuda")
    value = iters_all / total_dev_s

    # ---- the mixed FP32/FP64 form on the same workload (same protocol)
    mixed = None
    if not args.no_mixed:
        mopts = P.default_opts(allow_switch=0, max_iter=args.max_iter, precision=P.PREC_MIXED)
        for _ in range(min(1, args.warmup)):
            solver.reset_params()
            solver.levmar(mopts, fetch=False, trace_cap=0)
        m_ms, m_iters, m_costs = [], 0, []
        for _ in range(args.steps):
            solver.reset_params()
            flush_l2(torch, flush)
            r = solver.levmar(mopts, fetch=False, trace_cap=0)
            m_ms.append(r.device_ms)
            m_iters += r.iterations
            m_costs.append(r.final_cost)
        solver.set_stage_timing(True)  # the breakdown: one more solve with every stage timed
        solver.reset_params()
        solver.levmar(mopts, fetch=False, trace_cap=0)
        m_stages = solver.stage_timing()
        solver.set_stage_timing(False)
        mixed = {"value": m_iters / (sum(m_ms) / 1e3), "unit": UNIT, "ms_per_step": sum(m_ms) / len(m_ms),
                 "final_cost": m_costs[-1], "final_cost_rel_vs_fp64": abs(m_costs[-1] - costs[-1]) / costs[-1],
                 "speedup_vs_fp64": (m_iters / sum(m_ms)) / (iters / sum(dev_ms)),
                 "stage_ms": {k: (v[0] / v[1] if v[1] else 0.0) for k, v in m_stages.items()}}

    # ---- trust region (dogleg) on the same workload, FP64, same protocol
    tr = None
    if args.tr_iters > 0:
        topts = P.default_opts(allow_switch=0, max_iter=args.tr_iters)
        solver.reset_params()
        solver.trust_region(topts, fetch=False, trace_cap=0)  # warm-up
        t_ms, t_iters, t_cost = [], 0, None
        for _ in range(max(1, min(args.steps, 3))):
            solver.reset_params()
            flush_l2(torch, flush)
            r = solver.trust_region(topts, fetch=False, trace_cap=0)
            t_ms.append(r.device_ms)
            t_iters += r.iterations
            t_cost = r.final_cost
        tr = {"value": t_iters / (sum(t_ms) / 1e3), "unit": UNIT, "ms_per_step": sum(t_ms) / len(t_ms),
              "iterations_per_solve": t_iters / len(t_ms), "final_cost": t_cost,
              "driver": "trust_region (dogleg / 2-D subspace, modified-Cholesky fallback), FP64"}

    # ---- end to end through the C ABI from host buffers
    e2e_s, e2e_iters, h2d, d2h = 0.0, 0, 0, 0
    for _ in range(args.e2e_steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        with P.Solver(sc) as s2:
            r2 = s2.levmar(opts, fetch=True, trace_cap=0)
            a, b = s2.transfer_bytes()
        e2e_s += time.perf_counter() - t
        e2e_iters += r2.iterations
        h2d, d2h = a, b
    e2e_value = e2e_iters / e2e_s if e2e_s > 0 else None

    # ---- rooflines: the dominant kernel (k_schur), the dense solve and the whole Schur stage
    peak_gbs, peak_kind = measured_peaks()
    fp64_peak = P.measure_peak("fp64")
    schur_ms = sum(stages[k][0] for k in ("schur_off", "schur_diag", "schur_reduce"))
    schur_n = max(stages["schur_off"][1], 1)
    schur_avg_s = schur_ms / schur_n / 1e3
    achieved_gbs = schur_bytes(sc) / schur_avg_s / 1e9
    fp64_achieved = schur_flops(cfg) / schur_avg_s / 1e12
    chol_avg_s = live["cholesky"][0] / max(live["cholesky"][1], 1) / 1e3
    # k_schur (the "schur_off" stage: the diagonal units run in the same
    # launch): 6x6x3 FMAs per camera-pair entry and (21 + 6) x 3 per
    # observation; algorithmic bytes are Y and W of every observation (FP64),
    # the two pair-entry lists and the camera-sorted observation list
    soff_avg_s = live["schur_off"][0] / max(live["schur_off"][1], 1) / 1e3
    soff_flops = schur_flops(cfg)
    soff_bytes = 2 * sc.n_obs * 18 * 8 + 2 * 4 * cfg["pair_entries"] + 4 * sc.n_obs
    Np = -(-6 * sc.n_cams // 16) * 16
    chol_flops = Np ** 3 / 3 + 2 * Np ** 2
    chol_bytes = Np * Np * 8 + 2 * Np * 8
    stage_ms = {k: (v[0] / v[1] if v[1] else 0.0) for k, v in stages.items()}
    total_stage = sum(v[0] for v in stages.values())

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": sum(dev_ms) / len(dev_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": cfg, "parallelism": "replicas" if world > 1 else "single",
        "solves_per_s": len(dev_ms) * world / total_dev_s,
        "latency_ms": {"p50": float(np.percentile(dev_ms, 50)), "p99": float(np.percentile(dev_ms, 99))},
        "iterations_per_solve": iters / len(dev_ms), "trials_per_solve": trials / len(dev_ms),
        "final_cost": costs[-1], "wall_ms_per_step": 1e3 * wall / args.steps,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "steps": args.e2e_steps},
        "roofline": {"kernel": "k_schur: off-diagonal and diagonal blocks of the Schur complement, one launch "
                               "per LM trial (the largest share of the launch list)",
                     "bound": "fp64", "achieved": soff_flops / soff_avg_s / 1e12, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": soff_flops / soff_avg_s / 1e12 / fp64_peak,
                     "peak_source": "measured FP64 FMA rate (psba_measure_peak); MEASURED_PEAKS.json "
                                    "carries no FP64 figure",
                     "traffic": SCHUR_TRAFFIC, "algorithmic_flops": soff_flops, "avg_ms": soff_avg_s * 1e3,
                     "hbm": {"achieved": soff_bytes / soff_avg_s / 1e9, "peak": peak_gbs, "unit": "GB/s",
                             "frac": soff_bytes / soff_avg_s / 1e9 / peak_gbs, "algorithmic_bytes": soff_bytes,
                             "peak_source": peak_kind}},
        "roofline_chol": {"kernel": "k_chol_dataflow + k_tri_cluster: Cholesky of S + mu I and the triangular "
                                    "solves, one pair of launches per LM trial, N = %d" % Np,
                     "bound": "fp64", "achieved": chol_flops / chol_avg_s / 1e12, "peak": fp64_peak,
                     "unit": "TFLOP/s", "frac": chol_flops / chol_avg_s / 1e12 / fp64_peak,
                     "peak_source": "measured FP64 FMA rate (psba_measure_peak); MEASURED_PEAKS.json "
                                    "carries no FP64 figure",
                     "traffic": CHOL_TRAFFIC, "algorithmic_flops": chol_flops, "avg_ms": chol_avg_s * 1e3,
                     "hbm": {"achieved": chol_bytes / chol_avg_s / 1e9, "peak": peak_gbs, "unit": "GB/s",
                             "frac": chol_bytes / chol_avg_s / 1e9 / peak_gbs, "algorithmic_bytes": chol_bytes,
                             "peak_source": peak_kind}},
        "roofline_schur": {"kernel": "schur (k_schur + k_schur_reduce), per trial",
                           "bound": "fp64", "achieved": fp64_achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                           "frac": fp64_achieved / fp64_peak, "flops": schur_flops(cfg),
                           "traffic": SCHUR_TRAFFIC, "traffic_kernel": "k_schur",
                           "avg_ms": schur_avg_s * 1e3,
                           "hbm": {"achieved": achieved_gbs, "peak": peak_gbs, "unit": "GB/s",
                                   "frac": achieved_gbs / peak_gbs, "algorithmic_bytes": schur_bytes(sc),
                                   "peak_source": peak_kind}},
        "stage_ms": stage_ms, "mixed": mixed, "trust_region": tr,
        "stage_share": {k: (v[0] / total_stage if total_stage else 0.0) for k, v in stages.items()},
        "clocks": clk, "gpu_launches": int(launches),
    }
    if rank == 0 and not args.no_cpu:
        cb, nthreads = cpu_baseline(sc, args)
        v, r, dt = cb["threads"]
        # the same iterations on the GPU for a cost comparison at equal iteration count
        with P.Solver(sc) as s3:
            g = s3.levmar(P.default_opts(allow_switch=0, max_iter=r.iterations), fetch=False, trace_cap=0)
        line["cpu_baseline"] = {
            "value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "%d LM iterations of the same problem (FP64 C oracle, OpenMP), %.1f s" % (r.iterations, dt),
            "single_thread_value": cb["single"][0],
            "cost_after_sample": r.final_cost, "gpu_cost_after_sample": g.final_cost,
            "cost_rel_diff": abs(g.final_cost - r.final_cost) / r.final_cost,
        }
    if rank == 0 and args.varcam_iters > 0:
        line["variable_intrinsics"] = varcam_leg(P, args)
    if rank == 0 and args.batch > 0:
        line["batched"] = batched_leg(P, args)
    if rank == 0 and args.serve_rates.strip() not in ("", "none"):
        line["serving"] = serving_leg(P, args)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

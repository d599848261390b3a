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
  FP64 FMA rate.  roofline_chol: the dense solve (k_chol_dataflow +
  k_tri_cluster); roofline_mixed: the mixed form's Schur products
  (k_schur_f32) against the FP32 FMA rate and HBM.
* matched_cost: solves at matched final cost, on the bench problem and
  more seeded problems of the same shape.  The FP64 form runs to the
  reference's own stopping rule (levmar.cpp:157-179, 247-248) from the
  initial estimate; its cost C* is the target.  Each form (FP64, mixed) is
  then timed to the first iteration whose cost is within 1e-6 of C* (the
  same trajectory cut at that iteration), and the mixed form's own
  converged endpoint is reported with an FP64 polish from it.  LM on these
  problems (2% outliers) is chaotic past ~20 iterations, so which of
  several minima a trajectory ends in changes with its last bits; a
  problem where the mixed form ends in another minimum (certified by the
  polish) has no matched time, and the summary counts both kinds.  The
  control: the FP64 form from the initial estimate with the points moved by
  one ulp, and whether it ends in the same minimum as unmoved.
* refine: one FP64 solve of the same budget with the refinement step of
  the reduced solve on (psba_opts.refine), its dense-solve stage timed.
* variable_intrinsics: 52 cameras x 64,053 points with 11- and
  16-parameter cameras, the same matched-cost protocol.
* batched: 1,024 small problems in one persistent launch, every problem
  solved to the reference's stopping rule (mixed form, autotuned shape)
  against the plain FP64 single-problem solver doing the same problem by
  problem; final costs against the FP64 ones.
* serving: Poisson arrivals into the continuous-batching server (batch lane
  plus large lane), each request solved to the stopping rule; solves/s,
  p50/p99 latency per arrival rate, against the plain FP64 solver on the
  same request sequence.
* cpu_baseline: the FP64 CPU oracle (a C restatement of the reference's
  path) on the host cores: the same 50-iteration solve on all cores, a
  5-iteration sample on one.
* --impl reference: the CPU oracle alone (the reference's OpenCL/MSVC path
  does not build on this machine), the same 50-iteration solve per step.
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

# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch, from
# one ncu capture of this workload's kernels.
SCHUR_TRAFFIC = 250.1e6
CHOL_TRAFFIC = 1.30e6  # S (2.2 MB) stays in L2 between the Schur stage and the factor
SCHUR_F32_TRAFFIC = 83.1e6  # k_schur_f32, mixed form: 79.8 MB read + 3.3 MB written
MATCH_TOL = 1e-6  # matched final cost: within 1e-6 relative of the FP64 converged cost


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--points", type=int, default=64298)
    ap.add_argument("--cams", type=int, default=88)
    ap.add_argument("--max-iter", type=int, default=50)
    ap.add_argument("--cpu-single-iters", type=int, default=5, help="oracle LM iterations of the one-thread sample")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--converge-cap", type=int, default=400,
                    help="iteration cap of the solves to the stopping rule (matched-cost legs)")
    ap.add_argument("--no-mixed", action="store_true", help="skip the mixed-form and matched-cost legs")
    ap.add_argument("--no-matched", action="store_true", help="skip the matched-cost leg")
    ap.add_argument("--matched-seeds", default="0,1,2,3",
                    help="problem seeds of the matched-cost leg (0: the bench problem)")
    ap.add_argument("--no-refine", action="store_true", help="skip the refinement-step leg")
    ap.add_argument("--tr-iters", type=int, default=50, help="trust-region leg iterations (0: skip)")
    ap.add_argument("--varcam", action="store_true", default=True)
    ap.add_argument("--no-varcam", dest="varcam", action="store_false", help="skip the variable-intrinsics leg")
    ap.add_argument("--batch", type=int, default=1024, help="problems in the batched leg (0: skip)")
    ap.add_argument("--batch-steps", type=int, default=3)
    ap.add_argument("--batch-cap", type=int, default=240, help="iteration cap of the batched and serving solves")
    ap.add_argument("--batch-handoff", type=int, default=48,
                    help="batched leg: iterations after which an unfinished problem moves to the single-problem "
                         "solver (0: skip)")
    ap.add_argument("--pbp-sample", type=int, default=64,
                    help="problems solved one by one by the plain FP64 form for the batched comparison")
    ap.add_argument("--serve-rates", default="50,200,1000,2000", help="Poisson rates, req/s ('none' to skip)")
    ap.add_argument("--serve-seconds", type=float, default=2.0, help="arrival window per rate")
    ap.add_argument("--serve-max", type=int, default=400, help="requests per rate at most")
    ap.add_argument("--serve-pool", type=int, default=32, help="distinct request scenes (cycled)")
    ap.add_argument("--serve-large-lanes", type=int, default=None, help="server large_lanes (default: library's)")
    ap.add_argument("--serve-large-obs", type=int, default=None, help="server large_obs (default: library's)")
    ap.add_argument("--serve-large-cams", type=int, default=None, help="server large_cams (default: library's)")
    ap.add_argument("--serve-large-chol", type=int, default=None,
                    help="server large_chol_ctas (default: library's)")
    ap.add_argument("--serve-fp64-intrinsics", type=int, default=None, choices=[0, 1],
                    help="server fp64_intrinsics: 11/16-parameter requests in FP64 (default: library's)")
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


def stage_rooflines(sc, cfg, stage_ms, real_bytes, peak_gbs, fp64_peak, fp32_peak=None):
    """Every per-trial or per-iteration stage against HBM and its compute
    pipe: algorithmic bytes of the stage's defined inputs and outputs (the
    scope table's formulas with the run's O, P, C and c = 6; real_bytes 8 for
    the FP64 form, 4 for the mixed form's FP32 arrays; the stages this design
    adds or splits -- V^-1, eb/dpb, the trial cost -- by the same rule) and
    its approximate FMA count (from the kernel's arithmetic), over the
    stage's CUDA-event time."""
    O, P, C, c, s = sc.n_obs, sc.n_pts, sc.n_cams, 6, real_bytes
    pairs = cfg["pair_entries"]
    st = {
        # J: the residual and the chain-rule Jacobian (k_cam_tables, k_linearize)
        "linearize": (O * (16 + 8) + P * 24 + C * (c + 9) * 8 + O * (2 * c + 6 + 2) * s, 110 * O),
        # U/V/W/g: W is written by the linearization here, so it is counted there
        "point_blocks": (O * (6 + 2) * s + O * 8 + P * 9 * 8 + 3 * P * 8, 18 * O),
        "camera_blocks": (O * (12 + 2) * s + O * 4 + C * c * c * 8 + C * c * 8, 54 * O),
        "vinv": (P * 6 * 8 * 2, 40 * P),
        "yblocks": (2 * O * 3 * c * s + P * 9 * s + O * 4, 54 * O),
        "schur_off": (2 * O * 3 * c * s + O * 4 + (C * c) ** 2 * 8, 108 * pairs + 81 * O),
        "eb_dpb": (O * 3 * c * s + O * 4 + (C * c + 3 * P) * 8 * 3 + P * 6 * 8, 18 * O + 9 * P),
        "trial_cost": (O * (16 + 8) + P * 24 * 2 + C * 17 * 8, 30 * O),
    }
    out = {}
    for k, (nbytes, fma) in st.items():
        t = stage_ms.get(k, 0.0)
        if t <= 0:
            continue
        gbs = nbytes / (t * 1e-3) / 1e9
        tf = 2 * fma / (t * 1e-3) / 1e12
        out[k] = {"ms": t, "algorithmic_bytes": int(nbytes), "hbm_gbs": gbs, "hbm_frac": gbs / peak_gbs,
                  "fma": int(fma), "tflops": tf}
        if fp32_peak:  # the mixed form: its products are FP32
            out[k]["fp32_frac"] = tf / fp32_peak
        else:
            out[k]["fp64_frac"] = tf / fp64_peak
    return out


def flush_l2(torch, buf):
    buf.zero_()
    torch.cuda.synchronize()


def cpu_baseline(sc, args):
    """The FP64 CPU oracle on the host cores: the bench's own solve (the same
    problem, the same iteration budget, from the same initial estimate) on
    every core, a bounded sample of it on one core, and (untimed) the same
    solve from the points moved by one ulp: LM on this problem is chaotic
    past ~20 iterations (2% outliers), so that spread is the yardstick for
    comparing 50-iteration costs."""
    import oracle
    nthreads = os.cpu_count() or 1
    sess = oracle.Session(sc)
    out = {}
    try:
        for tag, th, iters in (("threads", nthreads, args.max_iter), ("single", 1, args.cpu_single_iters)):
            o = oracle.default_opts(allow_switch=0, max_iter=iters, n_threads=th)
            t = time.perf_counter()
            r = sess.levmar(o, trace_cap=4096)
            dt = time.perf_counter() - t
            out[tag] = (r.iterations / dt, r, dt)
        o = oracle.default_opts(allow_switch=0, max_iter=args.max_iter, n_threads=nthreads)
        out["ulp"] = sess.levmar(o, pts=np.nextafter(sc.pts, np.inf), trace_cap=4096)
    finally:
        sess.close()
    return out, nthreads


def cost_after(trace, n_iter):
    """The cost after the first n_iter LM iterations, from a trace."""
    acc = trace[(trace["accepted"] == 1) & (trace["itno"] < n_iter)]
    return float(acc["cost"][-1]) if len(acc) else float("nan")


def run_reference(args):
    """The reference arm: the FP64 CPU restatement of the reference's path on
    every host core, each step the same solve as ours (the same problem,
    the same iteration budget, from the initial estimate)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    import oracle
    from psba_gb300 import scenes
    sc = scenes.circle_scene(seed=0, n_cams=args.cams, n_pts=args.points, name="circle")
    cfg = workload_config(args, sc)
    nthreads = os.cpu_count() or 1
    sess = oracle.Session(sc)
    o = oracle.default_opts(allow_switch=0, max_iter=args.max_iter, n_threads=nthreads)
    for _ in range(args.warmup):
        sess.levmar(o)
    t = time.perf_counter()
    iters, step_s, cost = 0, [], None
    for _ in range(args.steps):
        t1 = time.perf_counter()
        r = sess.levmar(o)
        step_s.append(time.perf_counter() - t1)
        iters += r.iterations
        cost = r.final_cost
    dt = time.perf_counter() - t
    sess.close()
    value = iters / dt
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded generator)",
        "config": cfg, "impl": "reference",
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": nthreads, "kind": "port",
                         "sample": "the full solve of the workload per step (%d LM iterations from the initial "
                                   "estimate, FP64 C oracle, OpenMP), %d steps" % (args.max_iter, args.steps)},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "final_cost": cost, "latency_ms": {"p50": 1e3 * float(np.percentile(step_s, 50)),
                                           "p99": 1e3 * float(np.percentile(step_s, 99))},
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


def first_iteration_at(trace, target):
    """Outer LM iterations needed to reach cost <= target (from a trace), or None."""
    acc = trace[trace["accepted"] == 1]
    hit = acc[acc["cost"] <= target]
    return int(hit["itno"][0]) + 1 if len(hit) else None


def timed_cut(P, torch, flush, solver, precision, k, reps):
    """The form's solve from the initial estimate cut at iteration k (the
    same trajectory as its full run, which is deterministic): device ms
    (median of reps), trials and cost there."""
    o = P.default_opts(allow_switch=0, max_iter=k, precision=precision)
    ms = []
    for _ in range(max(1, reps)):
        solver.reset_params()
        flush_l2(torch, flush)
        r = solver.levmar(o, fetch=False, trace_cap=0)
        ms.append(r.device_ms)
    m = float(np.median(ms))
    return {"iterations": k, "trials": r.n_trials, "cost": r.final_cost, "ms": m, "solves_per_s": 1e3 / m,
            "iterations_per_s": k / (m / 1e3)}


def predictability_horizon(trace_ref, trace_ctl, tol=MATCH_TOL):
    """The last outer iteration k >= 1 up to which the costs of a run and of
    its control (the same run with the points moved by one ulp) agree to tol
    relative, and the run's cost there; (0, None) if they part at once."""
    cr, cn = cost_by_iteration(trace_ref), cost_by_iteration(trace_ctl)
    kh = 0
    for k in range(1, min(len(cr), len(cn))):
        if not abs(cr[k] - cn[k]) <= tol * cr[k]:
            break
        kh = k
    return (kh, float(cr[kh])) if kh > 0 else (0, None)


def summarize_matched(recs):
    """Summary over per-problem matched-cost records (matched_cost_leg): how
    many reached the FP64 converged cost in both forms, the speed-ups there
    and at the predictability horizon, and the other minima the mixed form
    ended in."""
    both = [r for r in recs if r["fp64"]["reached"] and r["mixed"]["reached"]]
    other = [r for r in recs if not r["mixed"]["reached"]]
    hz = [r["horizon"] for r in recs if "horizon" in r and "speedup_mixed_vs_fp64" in r["horizon"]]
    summary = {"problems": len(recs), "mixed_reached_fp64_minimum": len(both),
               "mixed_ended_in_another_minimum": len(other),
               "fp64_points_1ulp_same_minimum": sum(bool(r["fp64_points_1ulp"]["same_minimum"]) for r in recs)}
    if both:
        sp = [r["fp64"]["ms"] / r["mixed"]["ms"] for r in both]
        summary.update({
            "speedup_mixed_vs_fp64_geomean": float(np.exp(np.mean(np.log(sp)))),
            "speedup_mixed_vs_fp64_min": float(min(sp)), "speedup_mixed_vs_fp64_max": float(max(sp)),
            "fp64_ms_total": sum(r["fp64"]["ms"] for r in both),
            "mixed_ms_total": sum(r["mixed"]["ms"] for r in both)})
    if hz:
        sp = [h["speedup_mixed_vs_fp64"] for h in hz]
        summary["horizon"] = {
            "problems_reached": len(hz), "iterations": [h["iteration"] for h in hz],
            "speedup_mixed_vs_fp64_geomean": float(np.exp(np.mean(np.log(sp)))),
            "speedup_mixed_vs_fp64_min": float(min(sp)), "speedup_mixed_vs_fp64_max": float(max(sp)),
            "fp64_ms_total": sum(h["fp64"]["ms"] for h in hz), "mixed_ms_total": sum(h["mixed"]["ms"] for h in hz)}
    if other:
        summary["other_minima"] = [{"seed": r["seed"], "rel_vs_fp64": r["mixed"]["to_stopping_rule"]["rel_vs_fp64"],
                                    "fp64_polish_rel_decrease":
                                        r["mixed"]["to_stopping_rule"]["fp64_polish_rel_decrease"]}
                                   for r in other]
    return summary


def cost_by_iteration(trace):
    """cost[k] = the cost after k outer iterations (accepted steps only
    change it), from a trace; cost[0] is not recorded and stays NaN."""
    acc = trace[trace["accepted"] == 1]
    n = int(trace["itno"].max()) + 2 if len(trace) else 1
    c = np.full(n, np.nan)
    for it, cost in zip(acc["itno"], acc["cost"]):
        c[int(it) + 1] = cost
    for k in range(1, n):  # an iteration without an accepted step keeps the cost
        if np.isnan(c[k]) and k > 1:
            c[k] = c[k - 1]
    return c


def matched_cost_leg(P, torch, flush, sc, args, reps, solver=None):
    """Both forms on one problem at matched cost.  The FP64 form's run to the
    reference's stopping rule gives C*; the same run with the points moved by
    one ulp is the control.  Two targets:
      converged: within MATCH_TOL of C*; each form timed to its first
        iteration there (its trajectory cut at that iteration), the mixed
        form's own endpoint reported with an FP64 polish from it (FP64 LM
        restarted there: how much lower it gets);
      horizon: the FP64 cost at the last iteration where the FP64 run and its
        control still agree to MATCH_TOL (past it the trajectories' chaos,
        not their precision, decides where they go), each form timed to its
        first iteration within MATCH_TOL of it."""
    own = solver is None
    solver = solver or P.Solver(sc)
    try:
        cap = args.converge_cap
        runs = {}
        for tag, prec, nudge in (("fp64", P.PREC_FP64, False), ("mixed", P.PREC_MIXED, False),
                                 ("fp64_1ulp", P.PREC_FP64, True)):
            solver.reset_params()
            if nudge:
                cams0, pts0 = solver.get_params()
                solver.set_params(cams0, np.nextafter(pts0, np.inf))
            runs[tag] = solver.levmar(P.default_opts(allow_switch=0, max_iter=cap, precision=prec),
                                      fetch=(tag == "mixed"), trace_cap=50000)
        ref, mix, nud = runs["fp64"], runs["mixed"], runs["fp64_1ulp"]
        cstar = ref.final_cost
        out = {"target": {"cost": cstar, "tolerance": MATCH_TOL, "fp64_status": ref.status_name,
                          "fp64_iterations": ref.iterations, "cap": cap}}
        for tag, prec in (("fp64", P.PREC_FP64), ("mixed", P.PREC_MIXED)):
            full = runs[tag]
            res = {"to_stopping_rule": {"status": full.status_name, "iterations": full.iterations,
                                        "trials": full.n_trials, "final_cost": full.final_cost, "ms": full.device_ms}}
            k = first_iteration_at(full.trace, cstar * (1.0 + MATCH_TOL))
            res["reached"] = k is not None
            if k is not None:
                res.update(timed_cut(P, torch, flush, solver, prec, k, reps))
            out[tag] = res
        out["mixed"]["to_stopping_rule"]["rel_vs_fp64"] = (mix.final_cost - cstar) / cstar
        solver.set_params(mix.cams, mix.pts)
        pol = solver.levmar(P.default_opts(allow_switch=0, max_iter=100), fetch=False, trace_cap=0)
        out["mixed"]["to_stopping_rule"]["fp64_polish_rel_decrease"] = (mix.final_cost - pol.final_cost) / \
            pol.final_cost
        if out["fp64"]["reached"] and out["mixed"]["reached"]:
            out["speedup_mixed_vs_fp64"] = out["fp64"]["ms"] / out["mixed"]["ms"]
        out["fp64_points_1ulp"] = {"status": nud.status_name, "iterations": nud.iterations,
                                   "final_cost_rel_vs_fp64": (nud.final_cost - cstar) / cstar,
                                   "same_minimum": bool(abs(nud.final_cost - cstar) <= MATCH_TOL * cstar)}
        # the predictability horizon and the cost target there
        kh, th = predictability_horizon(ref.trace, nud.trace)
        if kh > 0:
            hz = {"iteration": kh, "cost": th}
            for tag, prec in (("fp64", P.PREC_FP64), ("mixed", P.PREC_MIXED)):
                k = first_iteration_at(runs[tag].trace, th * (1.0 + MATCH_TOL))
                hz[tag] = {"reached": k is not None}
                if k is not None:
                    hz[tag].update(timed_cut(P, torch, flush, solver, prec, k, reps))
            if hz["fp64"]["reached"] and hz["mixed"]["reached"]:
                hz["speedup_mixed_vs_fp64"] = hz["fp64"]["ms"] / hz["mixed"]["ms"]
            out["horizon"] = hz
        solver.reset_params()
        return out
    finally:
        if own:
            solver.close()


def matched_cost_instances(P, torch, flush, scenes, args, reps, solver):
    """The matched-cost protocol on several seeded problems of the bench's
    shape (seed 0 is the bench problem, on its solver): each problem's
    record, and a summary over the problems where both forms reached the
    FP64 target."""
    recs = []
    for seed in [int(x) for x in args.matched_seeds.split(",") if x.strip()]:
        if seed == 0:
            r = matched_cost_leg(P, torch, flush, None, args, reps, solver=solver)
        else:
            sc = scenes.circle_scene(seed=seed, n_cams=args.cams, n_pts=args.points, name="circle")
            r = matched_cost_leg(P, torch, flush, sc, args, reps)
        r["seed"] = seed
        recs.append(r)
    summary = summarize_matched(recs)
    return {"summary": summary, "problems": recs}


def batched_leg(P, args):
    """1,024 independent problems (5-30 cameras, 200-3,000 points, 3-8
    views) in one persistent launch under a CUDA graph, every problem solved
    to the reference's stopping rule (batch_cap iterations at most): the
    mixed form with the autotuned shape, the FP64 form in the same launch
    shape, and the plain FP64 single-problem solver one problem at a time on
    a sample of the same problems.  Also the configured fixed count (15
    iterations), which stops short of convergence."""
    from psba_gb300 import batch as B
    from psba_gb300 import scenes
    probs = scenes.batch_scenes(args.batch, seed=1000)
    cap = args.batch_cap
    mo = P.default_opts(allow_switch=0, max_iter=cap, precision=P.PREC_MIXED)
    fo = P.default_opts(allow_switch=0, max_iter=cap)

    def timed(b, o):
        b.reset()
        b.levmar(o)
        ms, res = [], None
        for _ in range(args.batch_steps):
            b.reset()
            res, t = b.levmar(o)
            ms.append(t)
        return res, float(np.median(ms))

    with B.Batch(probs) as b:
        choice, table = B.autotune(b, P.PREC_MIXED, iters=1, repeats=1)
        res_m, m_ms = timed(b, mo)
        res_f, f_ms = timed(b, fo)
        res_15, m15_ms = timed(b, P.default_opts(allow_switch=0, max_iter=15, precision=P.PREC_MIXED))
        res_15f, _ = timed(b, P.default_opts(allow_switch=0, max_iter=15))
        hand = None
        if args.batch_handoff > 0:
            ho_ms, ho = [], None
            for _ in range(args.batch_steps):
                b.reset()
                ho, bms, hms, todo = B.levmar_with_handoff(b, mo, args.batch_handoff)
                ho_ms.append((bms + hms, bms, hms, len(todo)))
            tot, bms, hms, nt = sorted(ho_ms)[len(ho_ms) // 2]
            rel_h = (ho["final_cost"] - res_f["final_cost"]) / res_f["final_cost"]
            hand = {"cap": args.batch_handoff, "handed_over": nt, "batch_ms": bms, "handoff_host_ms": hms,
                    "total_ms": tot, "mixed_solves_per_s": args.batch / (tot / 1e3),
                    "status": {P.STATUS_NAMES.get(int(k), str(k)): int(c)
                               for k, c in zip(*np.unique(ho["status"], return_counts=True))},
                    "frac_within_1e-6_of_fp64_converged": float((rel_h <= MATCH_TOL).mean()),
                    "note": "problems the persistent launch has not finished after `cap` iterations continue on "
                            "the single-problem solver from the batch's parameters and LM state "
                            "(psba_levmar_resume), up to 8 at once; batch device time plus the hand-over's "
                            "host time (handle creation included)"}
        dev_bytes = b.device_bytes()
    # the plain FP64 form, problem by problem (create outside the timing)
    sample = probs[: args.pbp_sample]
    pbp_ms, pbp_cost = [], []
    for sc in sample:
        with P.Solver(sc) as s:
            r = s.levmar(fo, fetch=False, trace_cap=0)
        pbp_ms.append(r.device_ms)
        pbp_cost.append(r.final_cost)
    pbp_cost = np.array(pbp_cost)
    cstar = res_f["final_cost"]
    rel = (res_m["final_cost"] - cstar) / cstar
    rel_pbp = (res_m["final_cost"][: len(sample)] - pbp_cost) / pbp_cost
    rel15 = (res_15["final_cost"] - cstar) / cstar
    m_sps = args.batch / (m_ms / 1e3)
    f_sps = args.batch / (f_ms / 1e3)
    pbp_sps = len(sample) / (sum(pbp_ms) / 1e3)
    st = np.unique(res_m["status"], return_counts=True)
    return {
        "workload": "%d problems, 5-30 cameras, 200-3,000 points, 3-8 views per point, each solved to the "
                    "reference's stopping rule (at most %d LM iterations), one persistent launch under a CUDA "
                    "graph" % (args.batch, cap),
        "observations": int(sum(sc.n_obs for sc in probs)), "device_bytes": int(dev_bytes),
        "mixed_solves_per_s": m_sps, "mixed_ms": m_ms,
        "mixed_iterations": {"mean": float(res_m["iterations"].mean()), "max": int(res_m["iterations"].max())},
        "mixed_status": {P.STATUS_NAMES.get(int(k), str(k)): int(c) for k, c in zip(*st)},
        "fp64_batched_solves_per_s": f_sps, "fp64_batched_ms": f_ms,
        "fp64_problem_by_problem_solves_per_s": pbp_sps,
        "fp64_problem_by_problem_sample": len(sample),
        "speedup_mixed_batched_vs_fp64_problem_by_problem": m_sps / pbp_sps,
        "handoff": hand,
        "speedup_mixed_handoff_vs_fp64_problem_by_problem": (hand["mixed_solves_per_s"] / pbp_sps) if hand else None,
        "matched": {"criterion": "final cost <= (1 + %g) x the FP64 converged cost of the same problem" % MATCH_TOL,
                    "frac_vs_fp64_batched": float((rel <= MATCH_TOL).mean()),
                    "frac_vs_fp64_problem_by_problem": float((rel_pbp <= MATCH_TOL).mean()),
                    "rel_max": float(rel.max()), "rel_min": float(rel.min()),
                    "rel_median_abs": float(np.median(np.abs(rel)))},
        "fp64_batched_vs_single_max_rel": float(np.max(np.abs(res_f["final_cost"][: len(sample)] - pbp_cost)
                                                       / pbp_cost)),
        "fixed_15_iterations": {"mixed_solves_per_s": args.batch / (m15_ms / 1e3),
                                "frac_within_1e-6_of_converged": float((np.abs(rel15) <= MATCH_TOL).mean()),
                                "fp64_mixed_rel_max": float(np.max(np.abs(res_15["final_cost"] - res_15f["final_cost"])
                                                                   / res_15f["final_cost"]))},
        "autotune": choice, "autotune_candidates": len(table),
    }


def varcam_leg(P, torch, flush, args):
    """Variable intrinsics: 52 cameras x 64,053 points (power-law views,
    mean 5.42), 11- and 16-parameter cameras, intrinsics 5% off: the
    matched-cost protocol of the single large problem, and LM iterations/s."""
    from psba_gb300 import scenes
    out = {}
    for cnp in (11, 16):
        sc = scenes.varcam_scene(cnp, seed=0)
        res = {"cameras": sc.n_cams, "points": sc.n_pts, "observations": sc.n_obs, "N": cnp * sc.n_cams}
        with P.Solver(sc) as s:
            res["matched_cost"] = matched_cost_leg(P, torch, flush, sc, args, 1, solver=s)
        out["cnp%d" % cnp] = res
    return out


def serving_leg(P, args):
    """Poisson arrivals of requests (cameras log-uniform 5-138, points
    500-60,000, 4-6 views, 6- or 11-parameter cameras) into the serving engine
    (mixed form for 6-parameter cameras, FP64 for cameras with intrinsics;
    every request solved to the reference's stopping rule, at most batch_cap
    iterations; 120 GB HBM budget); p50/p99 latency from submission to result
    on the host clock.  The baseline is the plain FP64 single-problem solver
    on the same request sequence, one request after another."""
    from psba_gb300 import scenes
    from psba_gb300 import serve as S
    rates = [float(x) for x in args.serve_rates.split(",") if x.strip()]
    pool = scenes.serving_scenes(args.serve_pool, seed=2000)
    # every other request scene with 11-parameter cameras (intrinsics 1% off)
    pool = [scenes.with_intrinsics(sc, 11, seed=3000 + q, k_off=0.01) if q % 2 else sc
            for q, sc in enumerate(pool)]
    cap = args.batch_cap
    # the plain FP64 form on each distinct scene: its converged cost and time
    fo = P.default_opts(allow_switch=0, max_iter=cap)
    pbp_ms, pbp_cost = [], []
    for sc in pool:
        with P.Solver(sc) as s:
            r = s.levmar(fo, fetch=False, trace_cap=0)
        pbp_ms.append(r.device_ms)
        pbp_cost.append(r.final_cost)
    out = {"workload": "Poisson arrivals; %d distinct request scenes cycled: cameras log-U[5,138], points "
                       "log-U[500,60000], 4-6 views/point, half 6-param and half 11-param cameras; each request "
                       "solved to the reference's stopping rule (at most %d LM iterations); mixed form for "
                       "6-param cameras, %s for 11-param; 120 GB HBM budget"
                       % (len(pool), cap, "mixed" if args.serve_fp64_intrinsics == 0 else "FP64"),
           "mean_observations": float(np.mean([sc.n_obs for sc in pool])), "rates": []}
    rel_all = []
    with S.Server(precision=P.PREC_MIXED, max_iter=cap, hbm_budget_bytes=120e9, large_cams=args.serve_large_cams,
                  large_lanes=args.serve_large_lanes, large_obs=args.serve_large_obs,
                  large_chol_ctas=args.serve_large_chol, fp64_intrinsics=args.serve_fp64_intrinsics) as srv:
        S.run_poisson(srv, pool[:4], rate=1000.0, n_requests=4, seed=1)
        for rate in rates:
            n = int(min(max(rate * args.serve_seconds, 20), args.serve_max))
            got, wall = S.run_poisson(srv, pool, rate, n, seed=int(rate))
            lat = np.array([r.latency_ms for r in got])
            qd = np.array([r.queued_ms for r in got])
            failed = [(q, r.status, r.error) for q, r in enumerate(got) if r.error is not None]
            rel = np.array([(r.final_cost - pbp_cost[q % len(pool)]) / pbp_cost[q % len(pool)]
                            for q, r in enumerate(got) if r.error is None])
            rel_all.append(rel)
            seq_ms = sum(pbp_ms[q % len(pool)] for q in range(n))
            out["rates"].append({"rate_req_s": rate, "requests": n, "solves_per_s": n / wall,
                                 "fp64_problem_by_problem_solves_per_s": n / (seq_ms / 1e3),
                                 "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99)),
                                 "queued_p50_ms": float(np.percentile(qd, 50)),
                                 "queued_p99_ms": float(np.percentile(qd, 99)),
                                 "matched_frac": float((rel <= MATCH_TOL).sum() / n),
                                 "failed_requests": len(failed),
                                 "failures": [{"request": q, "status": st, "error": msg} for q, st, msg in failed[:5]]})
        st = srv.stats()
    rel = np.concatenate(rel_all)
    best = max(out["rates"], key=lambda x: x["solves_per_s"])
    out["launches"] = st["launches"]
    out["peak_bytes"] = st["peak_bytes"]
    out["fp64_problem_by_problem_ms_mean"] = float(np.mean(pbp_ms))
    out["matched"] = {"criterion": "final cost <= (1 + %g) x the plain FP64 solver's on the same request" % MATCH_TOL,
                      "frac": float((rel <= MATCH_TOL).mean()), "rel_max": float(rel.max()),
                      "rel_min": float(rel.min())}
    out["speedup_vs_fp64_problem_by_problem"] = best["solves_per_s"] / best["fp64_problem_by_problem_solves_per_s"]
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

    # ---- the reduced solve with its refinement step (opts.refine): one FP64
    # solve of the same budget, the dense-solve stage timed
    refine = None
    if not args.no_refine:
        ropts = P.default_opts(allow_switch=0, max_iter=args.max_iter, refine=1)
        solver.set_stage_timing(True, stages=("cholesky",))
        solver.reset_params()
        flush_l2(torch, flush)
        r = solver.levmar(ropts, fetch=False, trace_cap=0)
        rs = solver.stage_timing()["cholesky"]
        solver.set_stage_timing(False)
        refine = {"value": r.iterations / (r.device_ms / 1e3), "unit": UNIT, "ms_per_step": r.device_ms,
                  "dense_solve_ms_per_trial": rs[0] / max(rs[1], 1),
                  "plain_dense_solve_ms_per_trial": live["cholesky"][0] / max(live["cholesky"][1], 1),
                  "final_cost": r.final_cost, "final_cost_rel_vs_plain": (r.final_cost - costs[-1]) / costs[-1],
                  "note": "residual as an accurate dot product against a copy of S, then both triangular "
                          "solves; FP64 form, same iteration budget"}

    # ---- the mixed FP32/FP64 form at the same iteration budget (same
    # protocol), with its Schur products (k_schur_f32) timed live
    mixed = None
    if not args.no_mixed:
        mopts = P.default_opts(allow_switch=0, max_iter=args.max_iter, precision=P.PREC_MIXED)
        for _ in range(min(1, args.warmup)):
            solver.reset_params()
            solver.levmar(mopts, fetch=False, trace_cap=0)
        solver.set_stage_timing(True, stages=("schur_off",))
        m_ms, m_iters, m_costs = [], 0, []
        for _ in range(args.steps):
            solver.reset_params()
            flush_l2(torch, flush)
            r = solver.levmar(mopts, fetch=False, trace_cap=0)
            m_ms.append(r.device_ms)
            m_iters += r.iterations
            m_costs.append(r.final_cost)
        m_live = solver.stage_timing()
        solver.set_stage_timing(True)  # the breakdown: one more solve with every stage timed
        solver.reset_params()
        solver.levmar(mopts, fetch=False, trace_cap=0)
        m_stages = solver.stage_timing()
        solver.set_stage_timing(False)
        mixed = {"value": m_iters / (sum(m_ms) / 1e3), "unit": UNIT, "ms_per_step": sum(m_ms) / len(m_ms),
                 "final_cost": m_costs[-1], "final_cost_rel_vs_fp64": (m_costs[-1] - costs[-1]) / costs[-1],
                 "note": "both forms stop at %d iterations, short of convergence, on different trajectories: "
                         "the cost comparison at matched final cost is matched_cost" % args.max_iter,
                 "speedup_vs_fp64": (m_iters / sum(m_ms)) / (iters / sum(dev_ms)),
                 "stage_ms": {k: (v[0] / v[1] if v[1] else 0.0) for k, v in m_stages.items()}}

    # ---- matched final cost: each form to within MATCH_TOL of the FP64 converged cost
    matched = None
    if not args.no_mixed and not args.no_matched:
        matched = matched_cost_instances(P, torch, flush, scenes, args, min(args.steps, 3), solver)

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
    # the FP64 tensor cores (mma.sync m8n8k4 / m16n8k16) against the FP64 FMA
    # rate: on GB300 they are slower, so no FP64 stage here uses them
    dmma = {"m8n8k4": P.measure_peak("dmma_m8n8k4"), "m16n8k16": P.measure_peak("dmma_m16n8k16"),
            "m8n8k4_and_fp64_fma_side_by_side": P.measure_peak("dmma_and_fp64"),
            "fp64_fma": fp64_peak, "unit": "TFLOP/s"}
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

    stage_roof = {"fp64": stage_rooflines(sc, cfg, stage_ms, 8, peak_gbs, fp64_peak),
                  "note": "per stage: the scope table's algorithmic bytes (O, P, C of this run; c = 6) and the "
                          "stage's approximate FMA count over its CUDA-event time; hbm_frac of the measured copy "
                          "rate, fp64_frac (FP64 form) or fp32_frac (mixed form) of the measured FMA rate.  Useful "
                          "FMAs only: a warp instruction costs the FP64 pipe the same with idle lanes, so the "
                          "pipe itself (ncu: sm__pipe_fp64_cycles_active) is busier than fp64_frac where lanes idle"}
    roofline_mixed = None
    if mixed is not None:
        fp32_peak = P.measure_peak("fp32")
        f32_s = m_live["schur_off"][0] / max(m_live["schur_off"][1], 1) / 1e3
        f32_bytes = 2 * sc.n_obs * 18 * 4 + 2 * 4 * cfg["pair_entries"] + 4 * sc.n_obs
        stage_roof["mixed"] = stage_rooflines(sc, cfg, mixed["stage_ms"], 4, peak_gbs, fp64_peak, fp32_peak)
        roofline_mixed = {
            "kernel": "k_schur_f32: the mixed form's Schur products (FP32 products, FP64 sums), off-diagonal "
                      "and diagonal units in one launch per LM trial",
            "bound": "l1", "avg_ms": f32_s * 1e3, "algorithmic_flops": soff_flops,
            "bound_note": "the L1 / shared-memory pipe (ncu: 87% of peak), not the FP32 pipe or HBM",
            "traffic": SCHUR_F32_TRAFFIC, "traffic_kernel": "k_schur_f32",
            "fp32": {"achieved": soff_flops / f32_s / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": soff_flops / f32_s / 1e12 / fp32_peak,
                     "peak_source": "measured FP32 FMA rate (psba_measure_peak)"},
            "hbm": {"achieved": f32_bytes / f32_s / 1e9, "peak": peak_gbs, "unit": "GB/s",
                    "frac": f32_bytes / f32_s / 1e9 / peak_gbs, "algorithmic_bytes": f32_bytes,
                    "peak_source": peak_kind}}

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
        "roofline_mixed": roofline_mixed, "stage_rooflines": stage_roof, "dmma_tflops": dmma,
        "stage_ms": stage_ms, "mixed": mixed, "matched_cost": matched, "trust_region": tr, "refine": refine,
        "stage_share": {k: (v[0] / total_stage if total_stage else 0.0) for k, v in stages.items()},
        "clocks": clk, "gpu_launches": int(launches),
    }
    if rank == 0 and not args.no_cpu:
        cb, nthreads = cpu_baseline(sc, args)
        v, r, dt = cb["threads"]
        v1, r1, dt1 = cb["single"]
        # the GPU's solve of the same budget, with its trace, against the oracle's
        solver.reset_params()
        g = solver.levmar(opts, fetch=False, trace_cap=4096)
        to, tg = r.trace[r.trace["itno"] < 10], g.trace[g.trace["itno"] < 10]
        c20o, c20g = cost_after(r.trace, 20), cost_after(g.trace, 20)
        line["cpu_baseline"] = {
            "value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": "the bench's solve (%d LM iterations from the initial estimate, FP64 C oracle, OpenMP on "
                      "%d threads), %.1f s" % (r.iterations, nthreads, dt),
            "single_thread_value": v1,
            "single_thread_sample": "%d LM iterations on one thread, %.1f s" % (r1.iterations, dt1),
            "parity": {
                "accept_sequence_first_10_iterations_equal": bool(
                    len(to) == len(tg) and np.array_equal(to["kind"], tg["kind"]) and
                    np.array_equal(to["accepted"], tg["accepted"])),
                "cost_after_20_iterations_rel_diff": abs(c20g - c20o) / c20o,
                "final_cost": r.final_cost, "gpu_final_cost": g.final_cost,
                "final_cost_rel_diff": abs(g.final_cost - r.final_cost) / r.final_cost,
                "oracle_final_cost_spread_1ulp_points": abs(cb["ulp"].final_cost - r.final_cost) / r.final_cost,
                "iterations_equal": bool(r.iterations == g.iterations),
                "note": "LM on this problem is chaotic past ~20 iterations: the oracle's own 50-iteration cost "
                        "moves by oracle_final_cost_spread_1ulp_points when the points move by one ulp"},
        }
    if rank == 0 and args.varcam:
        line["variable_intrinsics"] = varcam_leg(P, torch, flush, args)
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

"""Per-stage device times of an LM solve on a seeded scene.

``python -m psba_gb300.stages --precision mixed --iters 50`` solves the
88-camera circle scene (64,298 points, ~378k observations) with plain LM in
the chosen form: ``--reps`` solves for the iterations/s, then one more with
every stage bracketed by CUDA events, and prints each stage's mean time per
launch.  It is the command the per-stage ncu summaries are
captured under (a short ``--iters`` keeps the capture small).
"""
import argparse

from . import PREC_FP64, PREC_MIXED, Solver, default_opts
from . import scenes


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--precision", choices=("fp64", "mixed"), default="mixed")
    ap.add_argument("--iters", type=int, default=50, help="LM iteration cap of each solve")
    ap.add_argument("--reps", type=int, default=3, help="timed solves for the iterations/s")
    ap.add_argument("--cams", type=int, default=88)
    ap.add_argument("--points", type=int, default=64298)
    ap.add_argument("--seed", type=int, default=0)
    a = ap.parse_args(argv)
    sc = scenes.circle_scene(seed=a.seed, n_cams=a.cams, n_pts=a.points, name="circle")
    prec = PREC_MIXED if a.precision == "mixed" else PREC_FP64
    opts = default_opts(allow_switch=0, max_iter=a.iters, precision=prec)
    with Solver(sc) as s:
        s.reset_params()
        s.levmar(opts, fetch=False, trace_cap=0)  # warm-up
        ms, its = 0.0, 0
        for _ in range(a.reps):
            s.reset_params()
            r = s.levmar(opts, fetch=False, trace_cap=0)
            ms += r.device_ms
            its += r.iterations
        print("%s: %.1f LM it/s, final cost %.9e, %d trials" % (a.precision, its / ms * 1e3 if ms else 0.0,
                                                               r.final_cost, r.n_trials))
        s.set_stage_timing(True)
        s.reset_params()
        s.levmar(opts, fetch=False, trace_cap=0)
        st = s.stage_timing()
        s.set_stage_timing(False)
        for k, (tot, n) in st.items():
            if n:
                print("  %-13s %9.4f ms  x%d" % (k, tot / n, n))


if __name__ == "__main__":
    main()

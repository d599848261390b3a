"""CPU tests of bench.py's matched-cost bookkeeping: the iteration at which a
trace first reaches a cost, the cost after each outer iteration, the
predictability horizon between a run and its one-ulp control, and the
summary over problems.  These decide which speed-ups the bench reports, so
they are checked on hand-made traces."""
import math

import numpy as np

import bench
from psba_gb300 import TRACE_DTYPE


def trace(rows):
    """rows: (itno, accepted, cost) per trial record"""
    t = np.zeros(len(rows), dtype=TRACE_DTYPE)
    for k, (it, acc, cost) in enumerate(rows):
        t[k]["itno"], t[k]["accepted"], t[k]["cost"] = it, acc, cost
    return t


def test_first_iteration_at_counts_accepted_steps_only():
    t = trace([(0, 1, 10.0), (1, 0, 1.0), (1, 1, 8.0), (2, 1, 5.0)])
    assert bench.first_iteration_at(t, 9.0) == 2   # the rejected trial's 1.0 does not count
    assert bench.first_iteration_at(t, 5.0) == 3
    assert bench.first_iteration_at(t, 4.0) is None


def test_cost_by_iteration_carries_the_cost_over_rejected_iterations():
    t = trace([(0, 1, 10.0), (1, 0, 99.0), (2, 1, 7.0)])
    c = bench.cost_by_iteration(t)
    assert math.isnan(c[0])
    assert list(c[1:]) == [10.0, 10.0, 7.0]


def test_predictability_horizon_is_the_last_agreeing_iteration():
    ref = trace([(0, 1, 10.0), (1, 1, 8.0), (2, 1, 6.0), (3, 1, 5.0)])
    ctl = trace([(0, 1, 10.0), (1, 1, 8.0 * (1 + 5e-7)), (2, 1, 6.5), (3, 1, 5.0)])
    # agree to 1e-6 through iteration 2 (costs after 1 and 2 iterations), part at 3
    assert bench.predictability_horizon(ref, ctl, tol=1e-6) == (2, 8.0)
    assert bench.predictability_horizon(ref, ref, tol=1e-6) == (4, 5.0)
    apart = trace([(0, 1, 11.0)])
    assert bench.predictability_horizon(ref, apart, tol=1e-6) == (0, None)


def rec(seed, f_ms, m_ms, reached=True, same=False, horizon=None, rel=0.0):
    r = {"seed": seed, "fp64": {"reached": True, "ms": f_ms},
         "mixed": {"reached": reached, "ms": m_ms,
                   "to_stopping_rule": {"rel_vs_fp64": rel, "fp64_polish_rel_decrease": -1e-15}},
         "fp64_points_1ulp": {"same_minimum": same}}
    if horizon is not None:
        r["horizon"] = horizon
    return r


def test_summary_counts_minima_and_takes_geometric_means():
    hz = {"iteration": 50, "speedup_mixed_vs_fp64": 2.0, "fp64": {"ms": 20.0}, "mixed": {"ms": 10.0}}
    recs = [rec(0, 40.0, 20.0, horizon=hz, same=True), rec(1, 30.0, 15.0 / 4.0 * 2.0, horizon=hz),
            rec(2, 10.0, 5.0, reached=False, rel=3e-2)]
    s = bench.summarize_matched(recs)
    assert s["problems"] == 3 and s["mixed_reached_fp64_minimum"] == 2
    assert s["mixed_ended_in_another_minimum"] == 1 and s["fp64_points_1ulp_same_minimum"] == 1
    assert math.isclose(s["speedup_mixed_vs_fp64_geomean"], math.sqrt(2.0 * 4.0))
    assert s["speedup_mixed_vs_fp64_min"] == 2.0 and s["speedup_mixed_vs_fp64_max"] == 4.0
    assert s["horizon"]["problems_reached"] == 2 and s["horizon"]["iterations"] == [50, 50]
    assert s["other_minima"] == [{"seed": 2, "rel_vs_fp64": 3e-2, "fp64_polish_rel_decrease": -1e-15}]

"""Covariance-weighted residuals (psba_problem_desc.cov) on the GPU against
the FP64 oracle: the whitened residual and Jacobian, the LM accept/reject
sequence, and the mixed form's final cost.  The reference parses these
covariances (PSBA/readparams.cpp:272-282) but does not use them."""
import numpy as np
import pytest

import oracle
import psba_gb300 as P
from psba_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    P.build()


def rel(a, b):
    return np.abs(a - b).max() / max(1.0, np.abs(b).max())


@pytest.mark.parametrize("cnp", [6, 16])
def test_weighted_stages_match_oracle(cnp):
    sc = scenes.arc_scene(seed=11, n_cams=7, n_pts=300)
    if cnp > 6:
        sc = scenes.with_intrinsics(sc, cnp, seed=12)
    sc = scenes.with_covariance(sc, seed=13)
    pr = oracle.OracleProblem(sc)
    with P.Solver(sc) as s:
        ex, cost = s.eval_residual()
        e_o = oracle.residual(pr, sc.cams, sc.pts)
        assert rel(ex, e_o) <= 1e-12 and abs(cost - oracle.sumsq(e_o)) <= 1e-12 * cost
        JA, JB = s.eval_jacobian()
        JA_o, JB_o = oracle.jacobian(pr, sc.cams, sc.pts)
        assert rel(JA, JA_o) <= 1e-11 and rel(JB, JB_o) <= 1e-11
        U, V, W, g = s.eval_normal(1.0)
        U_o, V_o, W_o, g_o, _ = oracle.normal_blocks(pr, JA_o, JB_o, e_o, 1.0)
        assert rel(U, U_o) <= 1e-11 and rel(V, V_o) <= 1e-11 and rel(g, g_o) <= 1e-10


def test_weighted_levmar_fp64_matches_oracle():
    sc = scenes.with_covariance(scenes.arc_scene(seed=14, n_cams=7, n_pts=400), seed=15)
    o = oracle.levmar(sc, allow_switch=0, max_iter=10)
    with P.Solver(sc) as s:
        g = s.levmar(allow_switch=0, max_iter=10)
    assert [(t["kind"], t["accepted"]) for t in g.trace] == [(t["kind"], t["accepted"]) for t in o.trace]
    assert g.status == o.status and g.iterations == o.iterations
    assert abs(g.final_cost - o.final_cost) <= 1e-9 * o.final_cost


def test_weighting_changes_the_solution_as_expected():
    # scaling every covariance by s^2 scales the cost by 1/s^2 and leaves the
    # minimiser (and so the accept/reject sequence) unchanged
    base = scenes.with_covariance(scenes.arc_scene(seed=16, n_cams=6, n_pts=250), seed=17)
    scaled = base.copy()
    scaled.cov = base.cov * 4.0
    with P.Solver(base) as s1, P.Solver(scaled) as s2:
        r1 = s1.levmar(allow_switch=0, max_iter=8)
        r2 = s2.levmar(allow_switch=0, max_iter=8)
    assert abs(r2.final_cost * 4.0 - r1.final_cost) <= 1e-9 * r1.final_cost
    assert np.abs(r1.cams - r2.cams).max() <= 1e-8 * max(1.0, np.abs(r1.cams).max())

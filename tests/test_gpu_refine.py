"""The refinement step of the reduced solve (psba_opts.refine).

The reference inverts S explicitly (SPD_inv.cl) and multiplies once
(matVec_mul, cl_linearalg.cpp:19); this library solves with the Cholesky
factor and, on request, takes one step of iterative refinement: r = ea - S dpa
formed as an accurate dot product against a copy of S, then both triangular
solves of r with the factor, added into dpa.  Checked here:
  * at a damping that leaves S ill-conditioned (cond ~1e8), the refined dpa's
    forward error against the exact solution of the GPU's own S (a host
    solve refined with correctly rounded residuals) is at the rounding floor,
    below the plain solve's, in both precision forms and across the cluster
    solve's block ownership (N = 42 and N = 144, 3 and 9 blocks of 16);
  * LM with the step on reproduces the oracle's accept/reject sequence with
    final cost within 1e-9 (the plain solve's error is far below what the
    LM decisions see);
  * the batched engine refuses the option.
"""
import math

import numpy as np
import pytest
import scipy.linalg as sla

import oracle
import psba_gb300 as P
from psba_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    P.build()


def exact_residual(S, b, x):
    """b - S x with each row correctly rounded: the products split exactly
    (Veltkamp/Dekker), the row summed by math.fsum."""
    f = 134217729.0  # 2^27 + 1

    def split(a):
        c = f * a
        hi = c - (c - a)
        return hi, a - hi

    ah, al = split(S)
    xh, xl = split(x[None, :])
    p = S * x[None, :]
    e = ((ah * xh - p) + ah * xl + al * xh) + al * xl
    return np.array([math.fsum([b[i]] + list(-p[i]) + list(-e[i])) for i in range(len(b))])


def exact_solution(S, b):
    c = sla.cho_factor(S, lower=True)
    x = sla.cho_solve(c, b)
    for _ in range(3):
        x = x + sla.cho_solve(c, exact_residual(S, b, x))
    return x


def step_errors(sc, precision, mu_rel):
    """Forward errors of the plain and refined dpa at damping mu_rel * max
    diagonal of U and V."""
    errs, conds = [], []
    with P.Solver(sc) as s:
        s.set_precision(precision)
        U, V, _, _ = s.eval_normal(1.0)
        mu = mu_rel * max(np.abs(np.einsum("kii->ki", U)).max(), np.abs(np.einsum("kii->ki", V)).max())
        for refine in (0, 1):
            s.set_refine(refine)
            _, _, S, ea = s.eval_reduced(mu)
            st, dp = s.eval_step()
            assert st == 0
            S = np.tril(S) + np.tril(S, -1).T
            xs = exact_solution(S, ea)
            conds.append(np.linalg.cond(S))
            errs.append(np.linalg.norm(dp[: s.N] - xs) / np.linalg.norm(xs))
    return errs, conds


@pytest.mark.parametrize("precision", [P.PREC_FP64, P.PREC_MIXED])
@pytest.mark.parametrize("shape", ["arc7", "arc24"])
def test_refine_forward_error(shape, precision):
    sc = scenes.arc_scene(seed=0) if shape == "arc7" else scenes.arc_scene(seed=1, n_cams=24, n_pts=3000)
    (plain, refined), conds = step_errors(sc, precision, 1e-9)
    assert min(conds) > 1e7  # the regime refinement is for
    assert refined <= 1e-13, (plain, refined)
    assert refined <= plain, (plain, refined)


def test_refine_well_conditioned_keeps_solution():
    # at LM's first damping (tau = 1e-3) S is well conditioned: both solves
    # sit at the rounding floor
    sc = scenes.circle_scene(seed=1, n_cams=24, n_pts=3000, name="circle24")
    (plain, refined), _ = step_errors(sc, P.PREC_FP64, 1e-3)
    assert plain <= 1e-13 and refined <= 1e-13


@pytest.mark.parametrize("name", ["arc0", "circle24"])
def test_refine_levmar_matches_oracle(name):
    sc = scenes.small_lm_scene(0) if name == "arc0" else scenes.circle_scene(seed=1, n_cams=24, n_pts=3000,
                                                                             name="circle24")
    o = oracle.levmar(sc, allow_switch=0, max_iter=20)
    with P.Solver(sc) as s:
        g = s.levmar(allow_switch=0, max_iter=20, refine=1)
    to, tg = o.trace[o.trace["itno"] < 10], g.trace[g.trace["itno"] < 10]
    assert np.array_equal(to["kind"], tg["kind"]) and np.array_equal(to["accepted"], tg["accepted"])
    assert g.status == o.status
    assert abs(g.final_cost - o.final_cost) <= 1e-9 * o.final_cost


def test_refine_bad_value_and_batch_refused():
    sc = scenes.small_lm_scene(0)
    with P.Solver(sc) as s:
        with pytest.raises(P.PSBAError):
            s.set_refine(2)
        with pytest.raises(P.PSBAError):
            s.levmar(max_iter=2, refine=3)
    from psba_gb300.batch import Batch
    b = Batch([sc])
    try:
        with pytest.raises(P.PSBAError):
            b.levmar(max_iter=2, refine=1)
    finally:
        b.close()

"""Variable intrinsics (11- and 16-parameter cameras) on the GPU against the
FP64 oracle: every stage in the reference layouts, the LM accept/reject
sequence, and the mixed form's final cost.  The reference has no kernels for
these models (it fixes cnp = 6); the oracle's Jacobian for them is checked
against finite differences in tests/test_oracle.py."""
import numpy as np
import pytest

import oracle
import psba_gb300 as P
from psba_gb300 import scenes
from tr_envelope import assert_tr_trace_close, tr_envelope

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    P.build()


def scene(cnp, seed=3, n_cams=7, n_pts=300):
    return scenes.with_intrinsics(scenes.arc_scene(seed=seed, n_cams=n_cams, n_pts=n_pts), cnp, seed=seed + 2)


def rel(a, b):
    return np.abs(a - b).max() / max(1.0, np.abs(b).max())


@pytest.mark.parametrize("cnp", [11, 16])
def test_varcam_stages_match_oracle(cnp):
    sc = scene(cnp)
    pr = oracle.OracleProblem(sc)
    with P.Solver(sc) as s:
        ex, cost = s.eval_residual()
        e_o = oracle.residual(pr, sc.cams, sc.pts)
        assert rel(ex, e_o) <= 1e-12
        assert abs(cost - oracle.sumsq(e_o)) <= 1e-12 * cost
        JA, JB = s.eval_jacobian()
        JA_o, JB_o = oracle.jacobian(pr, sc.cams, sc.pts)
        assert JA.shape == (sc.n_obs, 2, cnp)
        assert rel(JA, JA_o) <= 1e-11 and rel(JB, JB_o) <= 1e-11
        U, V, W, g = s.eval_normal(1.0)
        U_o, V_o, W_o, g_o, _ = oracle.normal_blocks(pr, JA_o, JB_o, e_o, 1.0)
        assert rel(U, U_o) <= 1e-11 and rel(V, V_o) <= 1e-11 and rel(W, W_o) <= 1e-11
        assert rel(g, g_o) <= 1e-10
        mu = 1e-3 * max(np.abs(np.einsum("jkk->jk", U_o)).max(), 1.0)
        Vinv, Y, S, ea = s.eval_reduced(mu)
        Vinv_o = oracle.vinv(V_o, mu)
        Y_o = oracle.yblocks(pr, W_o, Vinv_o)
        S_o = oracle.schur(pr, U_o, mu, Y_o, W_o)
        ea_o = oracle.ea(pr, Y_o, g_o)
        assert rel(Y, Y_o) <= 1e-10
        assert rel(S, S_o) <= 1e-10 and rel(ea, ea_o) <= 1e-10
        st, dp = s.eval_step()
        assert st == 0
        stc, L = oracle.cholesky(S_o)
        assert stc == 0
        dpa_o = oracle.chol_solve(L, ea_o)
        eb_o, dpb_o = oracle.eb_dpb(pr, W_o, Vinv_o, g_o, dpa_o)
        N = cnp * sc.n_cams
        # S is built from differently rounded sums; its conditioning (intrinsics
        # and distortion columns next to the pose) amplifies that in the step
        assert rel(dp[:N], dpa_o) <= 1e-6 and rel(dp[N:], dpb_o) <= 1e-6
        x = np.random.default_rng(0).normal(size=N + 3 * sc.n_pts)
        assert rel(s.eval_jmultiply(x), oracle.jmultiply(pr, JA_o, JB_o, x)) <= 1e-11


@pytest.mark.parametrize("cnp", [11, 16])
def test_varcam_levmar_fp64_matches_oracle(cnp):
    sc = scene(cnp, seed=8)
    o = oracle.levmar(sc, allow_switch=0, max_iter=10, solve_mode=1)
    with P.Solver(sc) as s:
        g = s.levmar(allow_switch=0, max_iter=10)
    acc_o = [(t["kind"], t["accepted"]) for t in o.trace]
    acc_g = [(t["kind"], t["accepted"]) for t in g.trace]
    assert acc_g == acc_o
    assert g.status == o.status and g.iterations == o.iterations
    assert abs(g.final_cost - o.final_cost) <= 1e-9 * o.final_cost
    assert g.cams.shape == (sc.n_cams, cnp)
    assert rel(g.cams, o.cams) <= 1e-6


def test_varcam_mixed_matched_final_cost():
    # 11-parameter cameras with intrinsics 1% off: FP64 LM (oracle) converges
    # in ~70 iterations; the mixed form must reach the same cost within 1e-6.
    # (With 5% off, LM's mu I damping creeps along the intrinsics directions
    # for ~280 iterations in either precision.)
    sc = scenes.with_intrinsics(scenes.arc_scene(seed=9, n_cams=9, n_pts=500), 11, seed=11, k_off=0.01)
    o = oracle.levmar(sc, allow_switch=0, max_iter=150, solve_mode=1)
    assert o.status == P.ITER_DP_NO_CHANGE
    with P.Solver(sc) as s:
        g = s.levmar(allow_switch=0, max_iter=150, precision=P.PREC_MIXED)
    assert abs(g.final_cost - o.final_cost) <= 1e-6 * o.final_cost


def test_varcam_distortion_mixed_tracks_fp64():
    # 16-parameter cameras: LM has not converged after hundreds of
    # iterations in either precision (distortion adds flat directions); the
    # mixed form must follow the FP64 oracle's descent: after 150 iterations
    # its cost is within 2e-3 relative of the oracle's
    sc = scenes.with_intrinsics(scenes.arc_scene(seed=9, n_cams=9, n_pts=500), 16, seed=11, k_off=0.01)
    o = oracle.levmar(sc, allow_switch=0, max_iter=150, solve_mode=1)
    with P.Solver(sc) as s:
        g = s.levmar(allow_switch=0, max_iter=150, precision=P.PREC_MIXED)
    assert abs(g.final_cost - o.final_cost) <= 2e-3 * o.final_cost
    assert g.final_cost < 2e-3 * g.initial_cost


@pytest.mark.parametrize("cnp", [11, 16])
def test_varcam_trust_region_trace_matches_oracle(cnp):
    # no reference counterpart: the dogleg driver with 11/16-parameter
    # cameras, its lambda fallback running the 3x3-block modified Cholesky on
    # S padded to a multiple of 3 with an identity block
    # (N = 77 and 112 here, neither a multiple of 3).  With 16 parameters
    # the dogleg is so ill-conditioned that a 1-ulp change of the points
    # changes the oracle's own decisions after a few iterations, so the
    # trace is compared over the leading iterations where the nudged oracle
    # runs agree (at least 3) and the run's end only where they all agree
    sc = scene(cnp)
    assert (cnp * sc.n_cams) % 3 != 0
    o, n, env = tr_envelope(sc, 10)
    assert n >= 3
    with P.Solver(sc) as s:
        g = s.trust_region(max_iter=12)
    assert_tr_trace_close(o, g, n, env, same_end=n == 10)


@pytest.mark.parametrize("cnp", [11, 16])
def test_varcam_hybrid_matches_oracle(cnp):
    # LM hands over to the dogleg after five good steps, as for 6-parameter
    # cameras: the LM part and the hand-over iteration equal the oracle's.
    # The dogleg part is as sensitive as above (its end status differs even
    # between the oracle built here and on the GPU's host), so the end is
    # held to the same minimum: final cost within 1e-6, or ten times the
    # oracle's own spread when the points move by one ulp or S is solved
    # instead of inverted
    sc = scene(cnp)
    o = oracle.solve_hybrid(sc)
    spread = abs(oracle.solve_hybrid(sc, solve_mode=1).final_cost - o.final_cost) / o.final_cost
    for sign in (np.inf, -np.inf):
        sc2 = sc.copy()
        sc2.pts = np.nextafter(sc.pts, sign)
        spread = max(spread, abs(oracle.solve_hybrid(sc2).final_cost - o.final_cost) / o.final_cost)
    with P.Solver(sc) as s:
        g = s.solve_hybrid()
    first_tr = lambda t: int(np.argmax(t["kind"] >= P.TRACE_TR_TRIAL))
    k = first_tr(o.trace)
    assert k > 0 and first_tr(g.trace) == k
    assert np.array_equal(o.trace["kind"][:k], g.trace["kind"][:k])
    assert np.array_equal(o.trace["accepted"][:k], g.trace["accepted"][:k])
    assert o.trace["itno"][k] == g.trace["itno"][k]
    assert abs(g.final_cost - o.final_cost) <= max(10 * spread, 1e-6) * o.final_cost

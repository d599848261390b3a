"""The FP64 CPU oracle against the reference's own arithmetic.

Pinned two ways: against tests/golden (outputs of the reference's kernels,
generated by tests/golden/make_golden.py) everywhere, and live against the
reference compiled here when its sources are present.
"""
import numpy as np
import pytest

import oracle
import oracle.ref as ref
from psba_gb300 import scenes


def test_residual_and_jacobian_match_reference_kernels(golden):
    sc, z = golden
    pr = oracle.OracleProblem(sc)
    ex = oracle.residual(pr, sc.cams, sc.pts)
    assert np.array_equal(ex, z["ex"])  # same expressions, same grouping: bit-exact
    JA, JB = oracle.jacobian(pr, sc.cams, sc.pts)
    # independent derivation (chain rule) vs the reference's expanded form
    assert np.allclose(JA, z["JA"], rtol=1e-12, atol=1e-12 * np.abs(z["JA"]).max())
    assert np.allclose(JB, z["JB"], rtol=1e-12, atol=1e-12 * np.abs(z["JB"]).max())
    # the reference's CPU Jacobian equals its OpenCL one
    assert np.array_equal(z["cpu_JA"], z["JA"][:8]) and np.array_equal(z["cpu_JB"], z["JB"][:8])


@pytest.mark.parametrize("tag,coeff", [("c1", 1.0), ("c2", 2.0), ("cm2", -2.0)])
def test_normal_blocks_bit_exact(golden, tag, coeff):
    sc, z = golden
    pr = oracle.OracleProblem(sc)
    U, V, W, g, d = oracle.normal_blocks(pr, z["JA"], z["JB"], z["ex"], coeff)
    for name, arr in (("U", U), ("V", V), ("W", W), ("g", g), ("uvdiag", d)):
        assert np.array_equal(arr, z[name + "_" + tag]), name


def test_reduced_system_bit_exact(golden):
    sc, z = golden
    pr = oracle.OracleProblem(sc)
    mu = float(z["mu"])
    Vinv = oracle.vinv(z["V_c1"], mu)
    assert np.array_equal(Vinv, z["Vinv"])
    Y = oracle.yblocks(pr, z["W_c1"], Vinv)
    assert np.array_equal(Y, z["Y"])
    S = oracle.schur(pr, z["U_c1"], mu, Y, z["W_c1"])
    assert np.array_equal(S, np.tril(z["S"]))
    assert np.array_equal(oracle.ea(pr, Y, z["g_c1"]), z["ea"])


def test_back_substitution_and_jmultiply_bit_exact(golden):
    sc, z = golden
    pr = oracle.OracleProblem(sc)
    assert np.array_equal(oracle.matvec(z["Sinv"], z["ea"]), z["dpa"])
    eb, dpb = oracle.eb_dpb(pr, z["W_c1"], z["Vinv"], z["g_c1"], z["dpa"])
    assert np.array_equal(eb, z["eb"]) and np.array_equal(dpb, z["dpb"])
    jx = oracle.jmultiply(pr, z["JA"], z["JB"], z["jx_in"])
    dense = z["jx_dense"].reshape(sc.n_pts, sc.n_cams, 2)[sc.obs_pt, sc.obs_cam].ravel()
    assert np.array_equal(jx, dense)
    # every unobserved (point, camera) entry of the reference's dense J x is zero
    assert np.count_nonzero(z["jx_dense"]) <= 2 * sc.n_obs


def test_spd_inverse_matches_numpy(golden):
    sc, z = golden
    st, Sinv = oracle.spd_inverse(np.tril(z["S"]))
    assert st == 0
    assert np.allclose(Sinv, z["Sinv"], rtol=1e-10, atol=1e-12 * np.abs(z["Sinv"]).max())
    st, L = oracle.cholesky(np.tril(z["S"]))
    x = oracle.chol_solve(L, z["ea"])
    assert np.allclose(x, z["dpa"], rtol=1e-9, atol=1e-12 * np.abs(z["dpa"]).max())


def test_spd_inverse_reports_non_spd():
    A = np.eye(6)
    A[4, 4] = -1.0
    st, _ = oracle.spd_inverse(A)
    assert st == 1


@pytest.mark.skipif(not ref.available(), reason="reference sources not present")
def test_live_reference_on_fresh_scene():
    sc = scenes.arc_scene(seed=3, n_cams=9, n_pts=120, arc_deg=40)
    rng = np.random.default_rng(2)
    cams = sc.cams.copy()
    cams[:, :3] = rng.normal(0, 0.02, (sc.n_cams, 3))
    pr = oracle.OracleProblem(sc)
    assert np.array_equal(oracle.residual(pr, cams, sc.pts), ref.compute_exQT(sc, cams, sc.pts))
    JA, JB = ref.compute_jacobiQT(sc, cams, sc.pts)
    ex = ref.compute_exQT(sc, cams, sc.pts)
    o = oracle.normal_blocks(pr, JA, JB, ex, 1.0)
    r = ref.normal_blocks(sc, JA, JB, ex, 1.0)
    for a, b in zip(o, r):
        assert np.array_equal(a, b)
    mu = 1e-3 * r[4].max()
    Vinv_r, Y_r, S_r, ea_r = ref.trial(sc, r[0], r[1], r[2], r[3], mu)
    Vinv = oracle.vinv(r[1], mu)
    Y = oracle.yblocks(pr, r[2], Vinv)
    assert np.array_equal(Y, Y_r)
    assert np.array_equal(oracle.schur(pr, r[0], mu, Y, r[2]), np.tril(S_r))
    assert np.array_equal(oracle.ea(pr, Y, r[3]), ea_r)


def test_jacobian_matches_finite_differences():
    sc = scenes.arc_scene(seed=4, n_cams=5, n_pts=40)
    rng = np.random.default_rng(0)
    cams = sc.cams.copy()
    cams[:, :3] = rng.normal(0, 0.02, (sc.n_cams, 3))
    pr = oracle.OracleProblem(sc)
    JA, JB = oracle.jacobian(pr, cams, sc.pts)
    h = 1e-6
    for o in range(0, sc.n_obs, 7):
        j, i = sc.obs_cam[o], sc.obs_pt[o]
        for m in range(6):
            cp, cm = cams.copy(), cams.copy()
            cp[j, m] += h
            cm[j, m] -= h
            d = -(oracle.residual(pr, cp, sc.pts)[o] - oracle.residual(pr, cm, sc.pts)[o]) / (2 * h)
            assert np.allclose(d, JA[o, :, m], rtol=1e-5, atol=1e-3)
        for m in range(3):
            pp, pm = sc.pts.copy(), sc.pts.copy()
            pp[i, m] += h
            pm[i, m] -= h
            d = -(oracle.residual(pr, cams, pp)[o] - oracle.residual(pr, cams, pm)[o]) / (2 * h)
            assert np.allclose(d, JB[o, :, m], rtol=1e-5, atol=1e-3)


def test_levmar_converges_and_is_deterministic():
    sc = scenes.small_lm_scene(0)
    a = oracle.levmar(sc, allow_switch=0, max_iter=20)
    b = oracle.levmar(sc, allow_switch=0, max_iter=20)
    assert a.final_cost < 1e-2 * a.initial_cost
    assert np.array_equal(a.trace, b.trace)
    assert np.array_equal(a.cams, b.cams) and np.array_equal(a.pts, b.pts)
    # cost decreases over the accepted trials
    acc = a.trace[a.trace["accepted"] == 1]["cost"]
    assert np.all(np.diff(acc) <= 0)


def test_levmar_result_independent_of_threads():
    sc = scenes.small_lm_scene(1)
    a = oracle.levmar(sc, allow_switch=0, max_iter=8, n_threads=1)
    b = oracle.levmar(sc, allow_switch=0, max_iter=8, n_threads=4)
    assert np.array_equal(a.trace, b.trace)


def test_trust_region_and_hybrid_run():
    sc = scenes.small_lm_scene(2)
    t = oracle.trust_region(sc, max_iter=20)
    assert t.final_cost < t.initial_cost
    h = oracle.solve_hybrid(sc)
    assert h.final_cost < 1e-2 * h.initial_cost
    assert set(np.unique(h.trace["kind"])) <= {oracle.TR_LM_TRIAL, oracle.TR_LM_SOLVE_FAIL,
                                                oracle.TR_TR_TRIAL, oracle.TR_TR_PB_FAIL,
                                                oracle.TR_LM_STOP}


def test_cholmod_makes_matrix_positive_definite():
    rng = np.random.default_rng(0)
    n = 12
    Q = rng.normal(size=(n, n))
    A = Q @ np.diag(np.linspace(-1, 3, n)) @ Q.T  # indefinite
    L, E = oracle.cholmod(np.tril(A))
    L = np.tril(L)
    assert np.all(E >= -1e-9)
    assert np.allclose(L @ L.T, A + np.diag(E), atol=1e-8 * np.abs(A).max())


def test_cholmod_on_spd_is_plain_cholesky():
    rng = np.random.default_rng(1)
    n = 9
    Q = rng.normal(size=(n, n))
    A = Q @ Q.T + n * np.eye(n)
    L, E = oracle.cholmod(np.tril(A))
    assert np.allclose(np.tril(L), np.linalg.cholesky(A), atol=1e-10)
    assert np.allclose(E, 0.0, atol=1e-9)


@pytest.mark.parametrize("cnp", [11, 16])
def test_variable_intrinsics_jacobian_matches_finite_differences(cnp):
    # the 11- / 16-parameter camera models have no reference kernels: the
    # oracle's analytic Jacobian is checked column by column against central
    # differences of its residual (e = m - pi, so J = -de/dp)
    base = scenes.arc_scene(seed=3, n_cams=5, n_pts=120)
    sc = scenes.with_intrinsics(base, cnp, seed=5)
    pr = oracle.OracleProblem(sc)
    JA, JB = oracle.jacobian(pr, sc.cams, sc.pts)
    for j in range(sc.n_cams):
        sel = sc.obs_cam == j
        for k in range(cnp):
            h = 1e-6 * max(1.0, abs(sc.cams[j, k]))
            cp, cm = sc.cams.copy(), sc.cams.copy()
            cp[j, k] += h
            cm[j, k] -= h
            d = -(oracle.residual(pr, cp, sc.pts) - oracle.residual(pr, cm, sc.pts)) / (2 * h)
            ana = JA[sel][:, :, k]
            assert np.abs(d[sel] - ana).max() <= 1e-6 * max(1.0, np.abs(ana).max()), (j, k)
    for i in range(0, sc.n_pts, 17):
        sel = sc.obs_pt == i
        for k in range(3):
            pp, pm = sc.pts.copy(), sc.pts.copy()
            pp[i, k] += 1e-6
            pm[i, k] -= 1e-6
            d = -(oracle.residual(pr, sc.cams, pp) - oracle.residual(pr, sc.cams, pm)) / 2e-6
            ana = JB[sel][:, :, k]
            assert np.abs(d[sel] - ana).max() <= 1e-6 * max(1.0, np.abs(ana).max()), (i, k)


def test_variable_intrinsics_reduce_to_fixed_model():
    # with the fixed K copied into the parameters and no distortion, the
    # 11-parameter model gives the 6-parameter residual bit for bit and the
    # same pose / point Jacobian up to rounding
    sc6 = scenes.arc_scene(seed=4, n_cams=5, n_pts=100)
    sc11 = sc6.copy()
    sc11.cnp = 11
    sc11.cams = np.concatenate([sc6.cams, sc6.K], axis=1)
    p6, p11 = oracle.OracleProblem(sc6), oracle.OracleProblem(sc11)
    assert np.array_equal(oracle.residual(p6, sc6.cams, sc6.pts), oracle.residual(p11, sc11.cams, sc11.pts))
    A6, B6 = oracle.jacobian(p6, sc6.cams, sc6.pts)
    A11, B11 = oracle.jacobian(p11, sc11.cams, sc11.pts)
    assert np.allclose(A11[:, :, :6], A6, rtol=1e-13, atol=1e-12)
    assert np.allclose(B11, B6, rtol=1e-13, atol=1e-12)


@pytest.mark.parametrize("cnp", [11, 16])
def test_variable_intrinsics_levmar_recovers_truth(cnp):
    base = scenes.arc_scene(seed=6, n_cams=7, n_pts=300)
    sc = scenes.with_intrinsics(base, cnp, seed=7)
    r = oracle.levmar(sc, allow_switch=0, max_iter=40)
    # the fit reaches the noise floor: N(0, 0.5 px) per coordinate gives an
    # expected cost of 2 O 0.25 at the truth; allow twice that
    assert r.final_cost < 2.0 * (2 * sc.n_obs * 0.25)
    assert r.final_cost < 1e-3 * r.initial_cost

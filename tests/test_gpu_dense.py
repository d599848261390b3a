"""The dense reduced-camera solve and its device-side waits, through the C ABI.

* psba_eval_dense_solve runs the solver's own factor + back solve
  (k_chol_dataflow, k_tri_cluster) on a caller matrix: checked against
  numpy's solve at the sizes of the workloads (N = 42 .. 2,048), and the
  failure test of the reference (SPD_inv.cl:66-107: a non-positive or
  non-finite pivot gives status 1) on indefinite, NaN and subnormal-pivot
  matrices.
* psba_eval_pivot_reciprocal: the pivot chain's reciprocal (approximate
  reciprocal + one order-3 Householder step) within 1 ulp of the correctly
  rounded 1.0 / x over 2^-80 .. 2^80.
* psba_set_wait_limit: a handle whose waits are cut to one poll reports the
  stall as PSBA_ERR_STATE (the waits end, the kernels return), and the same
  handle solves bit-identically to a fresh one once the default is back.
"""
import numpy as np
import pytest

import psba_gb300 as P
from psba_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    P.build()


def spd(n, cond, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(n, n)))
    ev = np.geomspace(1.0, cond, n)
    A = (Q * ev) @ Q.T
    return 0.5 * (A + A.T)


@pytest.mark.parametrize("n", [42, 96, 528, 832, 2048])
def test_dense_solve_matches_numpy(n):
    A = spd(n, 1e6, n)
    b = np.random.default_rng(n + 1).normal(size=n)
    st, x = P.dense_solve(np.tril(A), b)
    assert st == 0
    ref = np.linalg.solve(A, b)
    # backward error at the FP64 level, forward error within cond * eps
    assert np.abs(A @ x - b).max() <= 1e-12 * np.abs(A).max() * np.abs(x).max()
    assert np.abs(x - ref).max() <= 1e-8 * np.abs(ref).max()


def test_dense_solve_bitwise_repeatable():
    A = spd(528, 1e4, 7)
    b = np.ones(528)
    st1, x1 = P.dense_solve(np.tril(A), b)
    st2, x2 = P.dense_solve(np.tril(A), b)
    assert st1 == st2 == 0 and np.array_equal(x1, x2)


def test_dense_solve_reports_failed_pivots():
    n = 96
    A = spd(n, 1e3, 3)
    b = np.ones(n)
    # indefinite: one negative eigenvalue
    B = A - 2.0 * np.outer(np.eye(n)[40], np.eye(n)[40]) * A[40, 40]
    assert P.dense_solve(np.tril(B), b)[0] == 1
    # a NaN below the diagonal
    C = A.copy()
    C[70, 12] = C[12, 70] = np.nan
    assert P.dense_solve(np.tril(C), b)[0] == 1
    # a positive but subnormal pivot (the reciprocal flushes subnormals)
    D = np.eye(n)
    D[5, 5] = 1e-310
    assert P.dense_solve(D, b)[0] == 1
    # a tiny normal pivot whose update makes the next one negative (no silent inf)
    E = np.eye(n)
    E[20, 20] = 1e-300
    E[21, 20] = E[20, 21] = 1.0
    st, x = P.dense_solve(np.tril(E), b)
    assert st == 1


def test_pivot_reciprocal_within_one_ulp():
    rng = np.random.default_rng(11)
    e = np.arange(-80, 81)
    m = rng.uniform(1.0, 2.0, size=(e.size, 64))
    x = np.ldexp(m, e[:, None]).ravel()
    x = np.concatenate([x, np.ldexp(1.0, e), np.ldexp(np.nextafter(2.0, 1.0), e),
                        np.ldexp(np.nextafter(1.0, 2.0), e)])
    y = P.pivot_reciprocal(x)
    ref = 1.0 / x  # correctly rounded
    ulps = np.abs(y.view(np.int64) - ref.view(np.int64))
    assert ulps.max() <= 1, (x[ulps.argmax()], y[ulps.argmax()], ref[ulps.argmax()])


def test_wait_limit_stall_is_reported_and_handle_recovers():
    sc = scenes.circle_scene(seed=3, n_cams=24, n_pts=2000, name="circle24")
    with P.Solver(sc) as fresh:
        want = fresh.levmar(allow_switch=0, max_iter=6)
    with P.Solver(sc) as s:
        s.set_wait_limit(1)  # every dependent task of the dense factor gives up at once
        with pytest.raises(P.PSBAError, match="wait budget"):
            s.levmar(allow_switch=0, max_iter=6)
        s.set_wait_limit(0)
        s.reset_params()
        got = s.levmar(allow_switch=0, max_iter=6)
    assert got.final_cost == want.final_cost
    assert np.array_equal(got.trace, want.trace)
    assert np.array_equal(got.cams, want.cams) and np.array_equal(got.pts, want.pts)

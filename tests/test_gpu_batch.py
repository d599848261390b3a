"""The batched solver (one persistent launch, one CTA per problem) against
the FP64 oracle, and the invariance of a problem's result to the batch it is
in.  Through the C ABI (psba_batch_*)."""
import numpy as np
import pytest

import oracle
import psba_gb300 as P
from psba_gb300 import batch as B
from psba_gb300 import scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    P.build()


def small_batch(n, seed=0):
    return scenes.batch_scenes(n, seed=seed, cams=(5, 14), pts=(200, 700), views=(3, 8))


def test_batch_fp64_matches_oracle():
    probs = small_batch(6, seed=1)
    with B.Batch(probs) as b:
        res, ms = b.levmar(allow_switch=0, max_iter=15)
        for q, sc in enumerate(probs):
            o = oracle.levmar(sc, allow_switch=0, max_iter=15)
            assert res["status"][q] == o.status, q
            assert res["iterations"][q] == o.iterations, q
            assert abs(res["initial_cost"][q] - o.initial_cost) <= 1e-12 * o.initial_cost
            assert abs(res["final_cost"][q] - o.final_cost) <= 1e-9 * o.final_cost, q
            cams, pts = b.get_params(q)
            assert np.abs(cams - o.cams).max() <= 1e-6 * max(1.0, np.abs(o.cams).max())


def test_batch_problem_result_independent_of_batch():
    probs = small_batch(5, seed=2)
    with B.Batch(probs) as b:
        res_all, _ = b.levmar(allow_switch=0, max_iter=10)
        p_all = [b.get_params(q) for q in range(len(probs))]
    for q in (0, 3):
        with B.Batch([probs[q]]) as one:
            r1, _ = one.levmar(allow_switch=0, max_iter=10)
            c1, x1 = one.get_params(0)
        assert r1["final_cost"][0] == res_all["final_cost"][q]
        assert np.array_equal(c1, p_all[q][0]) and np.array_equal(x1, p_all[q][1])


def test_batch_repeatable_after_reset():
    probs = small_batch(4, seed=3)
    with B.Batch(probs) as b:
        r1, _ = b.levmar(allow_switch=0, max_iter=8, precision=P.PREC_MIXED)
        b.reset()
        r2, _ = b.levmar(allow_switch=0, max_iter=8, precision=P.PREC_MIXED)
    assert np.array_equal(r1, r2)


def test_batch_mixed_matched_final_cost():
    probs = small_batch(4, seed=4)
    with B.Batch(probs) as b:
        res, _ = b.levmar(allow_switch=0, max_iter=40, precision=P.PREC_MIXED)
    for q, sc in enumerate(probs):
        o = oracle.levmar(sc, allow_switch=0, max_iter=40)
        assert abs(res["final_cost"][q] - o.final_cost) <= 1e-6 * o.final_cost, q


def test_batch_shape_knobs_keep_results():
    probs = small_batch(4, seed=5)
    with B.Batch(probs) as b:
        r0, _ = b.levmar(allow_switch=0, max_iter=10)
        for th, lanes in ((128, 8), (512, 16)):
            b.reset()
            b.set_threads(th)
            b.set_lanes(np.full(len(probs), lanes))
            r, _ = b.levmar(allow_switch=0, max_iter=10)
            assert np.array_equal(r["status"], r0["status"])
            assert np.allclose(r["final_cost"], r0["final_cost"], rtol=1e-9, atol=0)


def test_autotune_returns_a_valid_choice():
    probs = small_batch(12, seed=6)
    with B.Batch(probs) as b:
        choice, table = B.autotune(b, n_buckets=2, repeats=1)
        assert choice["threads"] in (128, 256, 512)
        assert all(v in (8, 16, 32, None) for v in choice["lanes_per_bucket"].values())
        res, _ = b.levmar(allow_switch=0, max_iter=5, precision=P.PREC_MIXED)
        assert np.all(res["final_cost"] < res["initial_cost"])


def test_levmar_resume_continues_a_batch_problem():
    # the batch stopped at 6 iterations hands its parameters and LM state
    # (mu, nu, |p|^2) to the single-problem solver, which continues to 15:
    # the same decisions and cost as the oracle's uninterrupted 15 iterations
    probs = small_batch(3, seed=5)
    with B.Batch(probs) as b:
        res, _ = b.levmar(allow_switch=0, max_iter=6)
        for q, sc in enumerate(probs):
            o = oracle.levmar(sc, allow_switch=0, max_iter=15)
            if res["status"][q] != P.ITER_CONTINUE:
                continue  # converged within the cap: nothing to hand over
            cams, pts = b.get_params(q)
            with P.Solver(sc) as s:
                s.set_params(cams, pts)
                g = s.levmar_resume(P.default_opts(allow_switch=0, max_iter=15), res["mu"][q], res["nu"][q],
                                    res["p_L2"][q], itno=int(res["iterations"][q]))
            assert g.status == o.status and g.iterations == o.iterations, q
            assert abs(g.final_cost - o.final_cost) <= 1e-9 * o.final_cost, q
            to = o.trace[o.trace["itno"] >= 6]
            assert np.array_equal(to["accepted"], g.trace["accepted"]), q


def test_levmar_resume_rejects_a_bad_state():
    sc = small_batch(1, seed=6)[0]
    with P.Solver(sc) as s:
        for mu, nu, pl2 in ((0.0, 2, 1.0), (1.0, 1, 1.0), (1.0, 2, float("nan"))):
            with pytest.raises(P.PSBAError):
                s.levmar_resume(P.default_opts(max_iter=3), mu, nu, pl2)


@pytest.mark.parametrize("precision", [P.PREC_FP64, P.PREC_MIXED])
def test_batch_handoff_matches_the_batch_alone(precision):
    # a low cap hands most problems over; every problem still ends at the
    # cost of the batch run to the stopping rule (FP64: to 1e-9; mixed: the
    # two engines' FP32 products differ, to 1e-6)
    probs = small_batch(12, seed=7)
    opts = P.default_opts(allow_switch=0, max_iter=240, precision=precision)
    with B.Batch(probs) as b:
        full, _ = b.levmar(opts)
        b.reset()
        got, batch_ms, hand_ms, todo = B.levmar_with_handoff(b, opts, cap=4, workers=4)
    assert len(todo) > 0 and batch_ms > 0 and hand_ms > 0
    assert np.all(got["status"] != P.ITER_CONTINUE)
    tol = 1e-9 if precision == P.PREC_FP64 else 1e-6
    rel = np.abs(got["final_cost"] - full["final_cost"]) / full["final_cost"]
    assert np.all(rel <= tol), rel

"""The serving engine (psba_server_*, psba_batch_submit/poll): continuous
batching with HBM-budget admission.  Results against the FP64 oracle, and the
same bits for a request alone and inside a stream of other requests."""
import time

import numpy as np
import pytest

import oracle
import psba_gb300 as P
from psba_gb300 import scenes
from psba_gb300 import serve as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def built():
    P.build()


def probs(n, seed):
    return scenes.batch_scenes(n, seed=seed, cams=(5, 16), pts=(200, 900), views=(3, 8))


def test_serve_fp64_matches_oracle():
    ps = probs(5, seed=11)
    with S.Server(precision=P.PREC_FP64, max_iter=12, hbm_budget_bytes=2e9) as srv:
        tickets = [srv.submit(sc) for sc in ps]
        res = [srv.wait(t) for t in tickets]
    for sc, r in zip(ps, res):
        o = oracle.levmar(sc, allow_switch=0, max_iter=12)
        assert r.status == o.status
        assert r.iterations == o.iterations
        assert abs(r.final_cost - o.final_cost) <= 1e-9 * o.final_cost
        assert np.abs(r.cams - o.cams).max() <= 1e-6 * max(1.0, np.abs(o.cams).max())


@pytest.mark.parametrize("precision", [P.PREC_FP64, P.PREC_MIXED])
def test_serve_same_bits_alone_and_in_mix(precision):
    ps = probs(9, seed=12)
    target = ps[4]
    with S.Server(precision=precision, max_iter=15, hbm_budget_bytes=2e9) as srv:
        alone = srv.wait(srv.submit(target))
    with S.Server(precision=precision, max_iter=15, hbm_budget_bytes=2e9, slice_iters=1) as srv:
        early = [srv.submit(sc) for sc in ps[:4]]
        time.sleep(0.02)  # the target arrives while the others are resident
        t = srv.submit(target)
        late = [srv.submit(sc) for sc in ps[5:]]
        mixed = srv.wait(t)
        for q in early + late:
            srv.wait(q)
        st = srv.stats()
    assert st["launches"] > 1
    assert mixed.final_cost == alone.final_cost
    assert mixed.iterations == alone.iterations and mixed.status == alone.status
    assert np.array_equal(mixed.cams, alone.cams) and np.array_equal(mixed.pts, alone.pts)


def test_serve_slice_length_does_not_change_results():
    ps = probs(4, seed=13)
    out = []
    for sl in (1, 4):
        with S.Server(precision=P.PREC_MIXED, max_iter=10, hbm_budget_bytes=2e9, slice_iters=sl) as srv:
            ts = [srv.submit(sc) for sc in ps]
            out.append([srv.wait(t) for t in ts])
    for a, b in zip(*out):
        assert a.final_cost == b.final_cost and np.array_equal(a.cams, b.cams)


def test_serve_admission_respects_budget():
    ps = probs(6, seed=14)
    # the pool holds the two largest problems at most
    with S.Server(precision=P.PREC_FP64, max_iter=6, hbm_budget_bytes=1e9, large_cams=0) as probe:
        sizes = [probe.wait(probe.submit(sc)).device_bytes for sc in ps]
    budget = sorted(sizes)[-1] + sorted(sizes)[-2] + 4096
    with S.Server(precision=P.PREC_FP64, max_iter=6, hbm_budget_bytes=budget, large_cams=0) as srv:
        ts = [srv.submit(sc) for sc in ps]
        res = [srv.wait(t) for t in ts]
        st = srv.stats()
    assert st["finished"] == len(ps)
    assert st["peak_bytes"] <= budget
    assert max(r.queued_ms for r in res) > 0.0
    for sc, r in zip(ps, res):
        o = oracle.levmar(sc, allow_switch=0, max_iter=6)
        assert abs(r.final_cost - o.final_cost) <= 1e-9 * o.final_cost


def test_serve_rejects_and_reports():
    big = scenes.batch_scenes(1, seed=15, cams=(20, 21), pts=(2000, 2001), views=(4, 6))[0]
    with S.Server(precision=P.PREC_FP64, max_iter=30, hbm_budget_bytes=2e6) as srv:
        with pytest.raises(P.PSBAError):
            srv.submit(big)  # alone larger than the pool: PSBA_ERR_NOMEM, nothing queued
        small = scenes.batch_scenes(1, seed=16, cams=(5, 5), pts=(200, 200), views=(3, 5))[0]
        t = srv.submit(small)
        r = srv.wait(t)
        assert r.status in (P.ITER_CONTINUE, P.ITER_DP_NO_CHANGE, P.ITER_ERR_SMALL_ENOUGH)
        with pytest.raises(KeyError):
            srv.poll(t)  # released by the successful poll


def test_serve_poisson_small():
    ps = probs(6, seed=17)
    with S.Server(precision=P.PREC_MIXED, max_iter=10, hbm_budget_bytes=2e9) as srv:
        out, wall = S.run_poisson(srv, ps, rate=200.0, n_requests=24, seed=3)
    assert all(r is not None for r in out)
    # the same scene gives the same bits whenever it arrived
    by_scene = {}
    for q, r in enumerate(out):
        by_scene.setdefault(q % len(ps), []).append(r.final_cost)
    for costs in by_scene.values():
        assert len(set(costs)) == 1
    assert wall > 0


@pytest.mark.parametrize("precision", [P.PREC_FP64, P.PREC_MIXED])
def test_serve_large_lane_in_a_mix(precision):
    # requests above large_cams run on the single-problem engine beside the
    # batch lane; their results are those of psba_levmar on the same problem
    small = probs(6, seed=18)
    large = [scenes.arc_scene(seed=19 + k, n_cams=46, n_pts=700, arc_deg=150.0, k_range=(3, 6),
                              name="large%d" % k) for k in range(2)]
    with S.Server(precision=precision, max_iter=12, hbm_budget_bytes=4e9, large_cams=40) as srv:
        ts = [srv.submit(sc) for sc in small[:3]] + [srv.submit(large[0])] + \
             [srv.submit(sc) for sc in small[3:]] + [srv.submit(large[1])]
        res = [srv.wait(t) for t in ts]
        st = srv.stats()
    assert st["finished"] == len(ts)
    for sc, r in zip(large, (res[3], res[-1])):
        with P.Solver(sc) as s:
            g = s.levmar(allow_switch=0, max_iter=12, precision=precision)
        assert r.final_cost == g.final_cost and r.iterations == g.iterations
        assert np.array_equal(r.cams, g.cams) and np.array_equal(r.pts, g.pts)
    for sc, r in zip(small, res[:3] + res[4:-1]):
        o = oracle.levmar(sc, allow_switch=0, max_iter=12)
        assert abs(r.final_cost - o.final_cost) <= (1e-9 if precision == P.PREC_FP64 else 1e-4) * o.final_cost


def test_serve_large_request_failure_is_its_own():
    # a large-lane solve whose device-side waits are cut to one poll gives up
    # (PSBA_ERR_STATE): poll reports that request as failed, with its error,
    # and the server goes on serving the batch lane beside it
    small = probs(3, seed=24)
    large = scenes.circle_scene(seed=3, n_cams=44, n_pts=2000, name="circle44")
    with S.Server(precision=P.PREC_FP64, max_iter=8, hbm_budget_bytes=4e9, large_cams=40,
                  large_wait_limit=1) as srv:
        tl = srv.submit(large)
        ts = [srv.submit(sc) for sc in small]
        r = srv.wait(tl)
        assert r.error is not None and "wait budget" in r.error
        assert r.status == P.PSBA_ERR_STATE
        res = [srv.wait(t) for t in ts]
        with pytest.raises(KeyError):
            srv.poll(tl)  # released
    for sc, got in zip(small, res):
        assert got.error is None
        o = oracle.levmar(sc, allow_switch=0, max_iter=8)
        assert abs(got.final_cost - o.final_cost) <= 1e-9 * o.final_cost


def test_serve_variable_intrinsics_and_weighted_requests():
    # 11-parameter cameras and covariance-weighted problems take the large
    # lane; their results are those of psba_levmar on the same problem
    base = scenes.arc_scene(seed=21, n_cams=8, n_pts=300)
    var11 = scenes.with_intrinsics(base, 11, seed=22, k_off=0.01)
    weighted = scenes.with_covariance(scenes.arc_scene(seed=23, n_cams=7, n_pts=250), seed=24)
    small = probs(3, seed=25)
    with S.Server(precision=P.PREC_FP64, max_iter=10, hbm_budget_bytes=4e9) as srv:
        ts = [srv.submit(var11), srv.submit(small[0]), srv.submit(weighted), srv.submit(small[1])]
        res = [srv.wait(t) for t in ts]
    for sc, r in ((var11, res[0]), (weighted, res[2])):
        with P.Solver(sc) as s:
            g = s.levmar(allow_switch=0, max_iter=10)
        assert r.final_cost == g.final_cost and np.array_equal(r.cams, g.cams)
    assert res[0].cams.shape == (8, 11)
    with S.Server(precision=P.PREC_FP64, max_iter=10, hbm_budget_bytes=4e9, large_cams=0) as srv:
        with pytest.raises(P.PSBAError):
            srv.submit(var11)  # no large lane to run it


@pytest.mark.parametrize("fp64_intrinsics", [1, 0])
def test_serve_mixed_server_precision_policy_for_intrinsics(fp64_intrinsics):
    # a mixed-precision server solves 11-parameter requests in FP64 unless
    # told otherwise: each result is psba_levmar's in the precision the
    # policy names
    var11 = scenes.with_intrinsics(scenes.arc_scene(seed=31, n_cams=8, n_pts=300), 11, seed=32, k_off=0.01)
    with S.Server(precision=P.PREC_MIXED, max_iter=10, hbm_budget_bytes=4e9,
                  fp64_intrinsics=fp64_intrinsics) as srv:
        r = srv.wait(srv.submit(var11))
    want = P.PREC_FP64 if fp64_intrinsics else P.PREC_MIXED
    with P.Solver(var11) as s:
        g = s.levmar(allow_switch=0, max_iter=10, precision=want)
    assert r.final_cost == g.final_cost and np.array_equal(r.cams, g.cams)

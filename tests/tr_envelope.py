"""The oracle's own spread over a trust-region trace, and the trace
comparison the GPU tests make against it (shared by the trust-region tests
of tests/test_gpu_parity.py and tests/test_gpu_varcam.py)."""
import numpy as np

import oracle
import psba_gb300 as P


def tr_envelope(sc, n_iter, max_iter=12, **okw):
    """The oracle's own spread over its trust-region trace when its inputs
    move by one ulp (points nudged up, points nudged down) or it solves
    instead of inverting S.  The reference's dogleg is ill-conditioned on
    these problems: its first Gauss-Newton step solves S + lambda I with S
    the singular lambda = 0 system (7 gauge directions) and lambda =
    |sum E| / N from the modified Cholesky of that singular S, so lambda moves
    by per cent and the early trial costs by ~1e-5 under a 1-ulp change of
    the input, while its LM path moves by 1e-15.  Returns the oracle's run,
    the number of leading iterations (at most n_iter) over which every nudged
    run makes the same decisions, and the per-record maximum relative spreads
    of cost and lambda over those iterations and that of the final cost.
    okw: further oracle options (n_threads)."""
    base = oracle.trust_region(sc, max_iter=max_iter, **okw)
    runs = []
    for sign in (np.inf, -np.inf):
        sc2 = sc.copy()
        sc2.pts = np.nextafter(sc.pts, sign)
        runs.append(oracle.trust_region(sc2, max_iter=max_iter, **okw))
    runs.append(oracle.trust_region(sc, max_iter=max_iter, solve_mode=1, **okw))
    n = n_iter
    while n > 0:
        t0 = base.trace[base.trace["itno"] < n]
        same = True
        for r in runs:
            t = r.trace[r.trace["itno"] < n]
            same = same and len(t) == len(t0) and np.array_equal(t["kind"], t0["kind"]) and \
                np.array_equal(t["accepted"], t0["accepted"])
        if same:
            break
        n -= 1
    t0 = base.trace[base.trace["itno"] < n]
    ec, el, ef = np.zeros(len(t0)), np.zeros(len(t0)), 0.0
    for r in runs:
        ef = max(ef, abs(r.final_cost - base.final_cost) / base.final_cost)
        t = r.trace[r.trace["itno"] < n]
        with np.errstate(invalid="ignore", divide="ignore"):
            ec = np.fmax(ec, np.abs(t["cost"] - t0["cost"]) / t0["cost"])
            el = np.fmax(el, np.abs(t["lambda_"] - t0["lambda_"]) / t0["lambda_"])
    return base, n, (np.nan_to_num(ec), np.nan_to_num(el), ef)


def assert_tr_trace_close(o, g, n_iter, env, same_end=True):
    """Over the first n_iter iterations: the record kinds (TR trials and the
    Gauss-Newton failures that send lambda through the modified Cholesky,
    trust_region.cpp:341-371), the accept decisions (trust_region.cpp:223-246)
    and the trust radius exactly; each trial's cost and lambda within ten
    times the oracle's own spread under 1-ulp input changes (plus 1e-9).
    With same_end (the nudged oracle runs agree over the whole run), also
    the status, the iteration count and the final cost likewise."""
    env_cost, env_lam, env_final = env
    to, tg = o.trace[o.trace["itno"] < n_iter], g.trace[g.trace["itno"] < n_iter]
    assert len(to) == len(tg)
    assert np.array_equal(to["itno"], tg["itno"])
    assert np.array_equal(to["kind"], tg["kind"]) and np.array_equal(to["accepted"], tg["accepted"])
    assert np.array_equal(to["damping"], tg["damping"])
    assert np.any(to["kind"] == P.TRACE_TR_PB_FAIL)  # the modified-Cholesky lambda path ran
    c = np.isfinite(to["cost"])
    assert np.array_equal(c, np.isfinite(tg["cost"]))
    dc = np.abs(tg["cost"][c] - to["cost"][c]) / to["cost"][c]
    assert np.all(dc <= 10 * env_cost[c] + 1e-9), (dc, env_cost[c])
    lam = to["lambda_"] > 0
    dl = np.abs(tg["lambda_"][lam] - to["lambda_"][lam]) / to["lambda_"][lam]
    assert np.all(dl <= 10 * env_lam[lam] + 1e-9), (dl, env_lam[lam])
    if same_end:
        assert g.status == o.status and g.iterations == o.iterations
        assert abs(g.final_cost - o.final_cost) <= (10 * env_final + 1e-9) * o.final_cost

"""The reference's own example problems through the GPU solver.

data/7camsvarK + 7pts (7 cameras, 465 points, 1,916 observations),
data/54camsvarK + 54pts (54, 5,207, 24,609) and Trafalgar-21-11315 (21,
11,315, 36,455; the problem PSBA/main.cpp:59-60 runs), read by this
repository's reader (pinned bit for bit to the reference's reader) and
carried in tests/golden/ref_data.npz.  Each is solved the way the
reference's main() sets it up (PSBA/main.cpp:102-149: K split off, the
rotation's vector part zeroed) by the GPU and by the FP64 oracle: LM
(levmar.cpp:45-256) must give the same accept/reject sequence over the
first 10 iterations and the same cost after 20 to 1e-9 (where LM
converged before that, the iteration its step-size test fires at may
differ: by then the step is rounding noise); the LM <-> TR alternation of
main.cpp:193-208 the same status and final cost to 1e-9.
"""
import numpy as np
import pytest

import oracle
import psba_gb300 as P

pytestmark = pytest.mark.gpu

COUNTS = {"7cams": (7, 465, 1916), "54cams": (54, 5207, 24609), "trafalgar21": (21, 11315, 36455)}


@pytest.fixture(scope="module", autouse=True)
def built():
    P.build()


@pytest.mark.parametrize("name", sorted(COUNTS))
def test_levmar_on_reference_problem(name, ref_data):
    sc = ref_data[name]
    assert (sc.n_cams, sc.n_pts, sc.n_obs) == COUNTS[name]
    o = oracle.levmar(sc, allow_switch=0, max_iter=20)
    with P.Solver(sc) as s:
        g = s.levmar(allow_switch=0, max_iter=20)
    to, tg = o.trace[o.trace["itno"] < 10], g.trace[g.trace["itno"] < 10]
    assert np.array_equal(to["kind"], tg["kind"]) and np.array_equal(to["accepted"], tg["accepted"])
    assert g.status == o.status
    # a run that converged stops when |dp|^2 < 1e-24 |p|^2 (levmar.cpp:157-164),
    # a test on a step that is rounding noise by then: the iteration it fires
    # at may differ; every other stop comes at the same iteration
    if o.status != P.ITER_DP_NO_CHANGE:
        assert g.iterations == o.iterations
    assert abs(g.initial_cost - o.initial_cost) <= 1e-12 * o.initial_cost
    assert abs(g.final_cost - o.final_cost) <= 1e-9 * o.final_cost
    assert g.final_cost < 0.1 * g.initial_cost


@pytest.mark.parametrize("name", sorted(COUNTS))
def test_hybrid_on_reference_problem(name, ref_data):
    sc = ref_data[name]
    o = oracle.solve_hybrid(sc)
    with P.Solver(sc) as s:
        g = s.solve_hybrid()
    assert g.status == o.status
    assert abs(g.final_cost - o.final_cost) <= 1e-9 * o.final_cost

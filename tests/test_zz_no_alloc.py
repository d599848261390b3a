"""psba_cost_noalloc: the reprojection cost for callers that cannot allocate
device memory (a stream being captured into a CUDA graph, a serving loop held
to a fixed HBM budget, a host framework that owns all device memory).  It
takes device arrays the caller already holds and uses a fixed scratch array
inside the library instead of cudaMalloc.

Checked through the C ABI against the existing entry point
(psba_eval_residual's cost) on two calls in a row, so a stale scratch from the
first call would show in the second; an observation index outside the
caller's point or camera range must be skipped on the device and reported as
a NaN cost.  This file is collected last.
"""
import ctypes as C

import numpy as np
import pytest

import psba_gb300 as P
from psba_gb300 import scenes

pytestmark = pytest.mark.gpu

TOL = 1e-10  # the FP64 stage tolerance of the other GPU parity tests


def _lib():
    P.build()
    L = P.lib()
    L.psba_cost_noalloc.argtypes = [C.c_int, C.c_int, C.c_int] + [C.c_void_p] * 9
    L.psba_cost_noalloc.restype = C.c_int
    return L


def _on_device(torch, a, dtype):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device="cuda")


def test_cost_noalloc_matches_eval_residual_twice():
    torch = pytest.importorskip("torch")
    L = _lib()
    sc = scenes.arc_scene(seed=21, n_cams=9, n_pts=400, arc_deg=40)
    rng = np.random.default_rng(3)
    for call in range(2):
        cams = sc.cams.copy()
        cams[:, :3] = rng.normal(0.0, 0.01, (sc.n_cams, 3))
        pts = sc.pts + rng.normal(0.0, 0.01, sc.pts.shape)
        with P.Solver(sc) as s:
            s.set_params(cams, pts)
            _, expected = s.eval_residual()
        d = {k: _on_device(torch, v, torch.float64)
             for k, v in dict(K=sc.K, q0=sc.q0, cams=cams, pts=pts, meas=sc.meas).items()}
        opt = _on_device(torch, sc.obs_pt, torch.int32)
        ocam = _on_device(torch, sc.obs_cam, torch.int32)
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        stream = torch.cuda.current_stream().cuda_stream
        rc = L.psba_cost_noalloc(sc.n_cams, sc.n_pts, sc.n_obs, d["K"].data_ptr(), d["q0"].data_ptr(),
                                 d["cams"].data_ptr(), d["pts"].data_ptr(), d["meas"].data_ptr(),
                                 opt.data_ptr(), ocam.data_ptr(), out.data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc == P.PSBA_OK, L.psba_last_error()
        got = out.item()
        assert abs(got - expected) <= TOL * expected, (call, got, expected)


def test_cost_noalloc_flags_out_of_range_indices():
    # the indices live in caller memory, so the kernel checks them: a point
    # index past n_pts or a negative camera index is skipped (no read through
    # it) and turns the cost into NaN; the valid call after it is unaffected
    torch = pytest.importorskip("torch")
    L = _lib()
    sc = scenes.arc_scene(seed=22, n_cams=5, n_pts=100)
    d = {k: _on_device(torch, v, torch.float64)
         for k, v in dict(K=sc.K, q0=sc.q0, cams=sc.cams, pts=sc.pts, meas=sc.meas).items()}
    stream = torch.cuda.current_stream().cuda_stream
    with P.Solver(sc) as s:
        _, expected = s.eval_residual()
    for bad_pt, bad_cam in ((sc.n_pts + 1000, None), (None, -3), (None, None)):
        opt_h, ocam_h = sc.obs_pt.copy(), sc.obs_cam.copy()
        if bad_pt is not None:
            opt_h[sc.n_obs // 2] = bad_pt
        if bad_cam is not None:
            ocam_h[7] = bad_cam
        opt = _on_device(torch, opt_h, torch.int32)
        ocam = _on_device(torch, ocam_h, torch.int32)
        out = torch.zeros(1, dtype=torch.float64, device="cuda")
        rc = L.psba_cost_noalloc(sc.n_cams, sc.n_pts, sc.n_obs, d["K"].data_ptr(), d["q0"].data_ptr(),
                                 d["cams"].data_ptr(), d["pts"].data_ptr(), d["meas"].data_ptr(),
                                 opt.data_ptr(), ocam.data_ptr(), out.data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc == P.PSBA_OK, L.psba_last_error()
        if bad_pt is None and bad_cam is None:
            assert abs(out.item() - expected) <= TOL * expected
        else:
            assert np.isnan(out.item())


def test_cost_noalloc_rejects_sizes_beyond_its_scratch():
    L = _lib()
    rc = L.psba_cost_noalloc(1025, 10, 10, 1, 1, 1, 1, 1, 1, 1, 1, None)
    assert rc == P.PSBA_ERR_ARG
    assert b"n_cams" in L.psba_last_error()
    rc = L.psba_cost_noalloc(4, 10, 1 << 25, 1, 1, 1, 1, 1, 1, 1, 1, None)
    assert rc == P.PSBA_ERR_ARG
    assert b"n_obs" in L.psba_last_error()
    rc = L.psba_cost_noalloc(4, -1, 10, 1, 1, 1, 1, 1, 1, 1, 1, None)
    assert rc == P.PSBA_ERR_ARG
    assert b"n_pts" in L.psba_last_error()

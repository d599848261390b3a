"""The C-ABI library: it builds for sm_103a, loads, exports every entry point
that include/psba.h declares, and rejects bad input before touching a GPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

import psba_gb300
from psba_gb300 import scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    names = set()
    for f in os.listdir(os.path.join(ROOT, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(psba_[a-z_0-9]+)\s*\(", txt))
    return names


@pytest.fixture(scope="module")
def L():
    psba_gb300.build()
    return psba_gb300.lib()


def test_exports_every_declared_symbol(L):
    syms = header_symbols()
    assert len(syms) >= 15
    assert syms == set(psba_gb300.EXPORTS)
    for s in syms:
        assert hasattr(L, s), s


def test_default_opts_are_reference_constants(L):
    o = psba_gb300.default_opts()
    assert o.tau == 1e-3 and o.stop_thresh == 1e-12 and o.eps == 1e-12 and o.eps2 == 1e-12
    assert o.max_iter == 50 and o.allow_switch == 1 and o.precision == psba_gb300.PREC_FP64
    assert o.refine == 0


def test_server_refuses_refine(L):
    # the refinement step is for the per-handle solver; the server's options
    # are checked before anything touches the device
    from psba_gb300.serve import Server
    with pytest.raises(psba_gb300.PSBAError):
        Server(refine=1)


def test_version_string(L):
    assert "sm_103a" in psba_gb300.version()


def _desc_args(sc):
    keep = [np.ascontiguousarray(a, dtype=np.float64) for a in (sc.K, sc.q0, sc.cams, sc.pts, sc.meas)]
    keep += [np.ascontiguousarray(sc.obs_pt, dtype=np.int32), np.ascontiguousarray(sc.obs_cam, dtype=np.int32)]
    return keep


def _create(L, sc, cnp=6):
    K, q0, cams, pts, meas, opt, ocam = keep = _desc_args(sc)
    d = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))  # noqa: E731
    desc = psba_gb300.ProblemDesc(sc.n_cams, sc.n_pts, sc.n_obs, d(K), d(q0), d(cams), d(pts), d(meas),
                                  opt.ctypes.data_as(C.POINTER(C.c_int)), ocam.ctypes.data_as(C.POINTER(C.c_int)),
                                  cnp)
    h = C.c_void_p()
    rc = L.psba_create(C.byref(desc), C.byref(h))
    del keep
    return rc, h


def test_create_rejects_unsorted_observations(L):
    sc = scenes.arc_scene(seed=0, n_cams=5, n_pts=20)
    bad = sc.copy()
    bad.obs_pt = bad.obs_pt[::-1].copy()
    bad.obs_cam = bad.obs_cam[::-1].copy()
    rc, h = _create(L, bad)
    assert rc == psba_gb300.PSBA_ERR_ARG and not h.value
    assert b"sorted" in L.psba_last_error()


def test_create_rejects_out_of_range_index(L):
    sc = scenes.arc_scene(seed=0, n_cams=5, n_pts=20)
    bad = sc.copy()
    bad.obs_cam = bad.obs_cam.copy()
    bad.obs_cam[-1] = 99
    rc, h = _create(L, bad)
    assert rc == psba_gb300.PSBA_ERR_ARG
    assert b"out of range" in L.psba_last_error()


def test_create_rejects_repeated_observation(L):
    sc = scenes.arc_scene(seed=0, n_cams=5, n_pts=20)
    bad = sc.copy()
    bad.obs_cam = bad.obs_cam.copy()
    bad.obs_cam[1] = bad.obs_cam[0]
    bad.obs_pt = bad.obs_pt.copy()
    bad.obs_pt[1] = bad.obs_pt[0]
    rc, _ = _create(L, bad)
    assert rc == psba_gb300.PSBA_ERR_ARG


def test_null_arguments(L):
    assert L.psba_create(None, None) == psba_gb300.PSBA_ERR_ARG
    h = C.c_void_p()
    assert L.psba_create(None, C.byref(h)) == psba_gb300.PSBA_ERR_ARG
    assert L.psba_eval_cholmod(4, None, None) == psba_gb300.PSBA_ERR_ARG


@pytest.mark.parametrize("cnp", [1, 7, 12, -6])
def test_create_rejects_unknown_camera_model(L, cnp):
    sc = scenes.arc_scene(seed=0, n_cams=5, n_pts=20)
    rc, h = _create(L, sc, cnp=cnp)
    assert rc == psba_gb300.PSBA_ERR_ARG and not h.value
    assert b"cnp" in L.psba_last_error()

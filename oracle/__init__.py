"""ctypes binding of the FP64 CPU oracle.  TEST INFRASTRUCTURE ONLY.

Only tests, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg
import this package, as the checker.  The product (``psba_gb300``) never
calls into it.
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

ITER_TURN_TO_LM, ITER_TURN_TO_TR, ITER_CONTINUE, ITER_ERR = 1, 2, 3, 4
ITER_DP_NO_CHANGE, ITER_ERR_SMALL_ENOUGH, ITER_PASS = 5, 6, 7
TR_LM_TRIAL, TR_LM_SOLVE_FAIL, TR_TR_TRIAL, TR_TR_PB_FAIL, TR_LM_STOP = 1, 2, 3, 4, 5

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class Problem(C.Structure):
    _fields_ = [("nc", C.c_int), ("np", C.c_int), ("no", C.c_int), ("K", _dp), ("q0", _dp),
                ("meas", _dp), ("obs_pt", _ip), ("obs_cam", _ip), ("cnp", C.c_int), ("wt", _dp)]


class Opts(C.Structure):
    _fields_ = [("tau", C.c_double), ("stop_thresh", C.c_double), ("eps", C.c_double),
                ("eps2", C.c_double), ("max_iter", C.c_int), ("allow_switch", C.c_int),
                ("solve_mode", C.c_int), ("n_threads", C.c_int)]


class Trace(C.Structure):
    _fields_ = [("itno", C.c_int), ("kind", C.c_int), ("accepted", C.c_int), ("pad", C.c_int),
                ("damping", C.c_double), ("rho", C.c_double), ("cost", C.c_double),
                ("lambda_", C.c_double)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("initial_cost", C.c_double),
                ("final_cost", C.c_double), ("n_trace", C.c_int), ("trace_cap", C.c_int),
                ("trace", C.POINTER(Trace))]


TRACE_DTYPE = np.dtype([("itno", np.int32), ("kind", np.int32), ("accepted", np.int32),
                        ("pad", np.int32), ("damping", np.float64), ("rho", np.float64),
                        ("cost", np.float64), ("lambda_", np.float64)])

_lib = None


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = C.CDLL(path)
        L.orc_default_opts.argtypes = [C.POINTER(Opts)]
        L.orc_residual.argtypes = [C.POINTER(Problem), _dp, _dp, _dp]
        L.orc_sumsq.argtypes = [C.c_int, _dp]
        L.orc_sumsq.restype = C.c_double
        L.orc_jacobian.argtypes = [C.POINTER(Problem), _dp, _dp, _dp, _dp]
        L.orc_normal_blocks.argtypes = [C.POINTER(Problem), _dp, _dp, _dp, C.c_double, _dp, _dp, _dp,
                                        _dp, _dp]
        L.orc_vinv.argtypes = [C.c_int, _dp, C.c_double, _dp]
        L.orc_yblocks.argtypes = [C.POINTER(Problem), _dp, _dp, _dp]
        L.orc_schur.argtypes = [C.POINTER(Problem), _dp, C.c_double, _dp, _dp, _dp]
        L.orc_ea.argtypes = [C.POINTER(Problem), _dp, _dp, _dp]
        L.orc_spd_inverse.argtypes = [C.c_int, _dp]
        L.orc_cholesky.argtypes = [C.c_int, _dp]
        L.orc_chol_solve.argtypes = [C.c_int, _dp, _dp, _dp]
        L.orc_matvec.argtypes = [C.c_int, _dp, _dp, _dp]
        L.orc_eb_dpb.argtypes = [C.POINTER(Problem), _dp, _dp, _dp, _dp, _dp, _dp]
        L.orc_jmultiply.argtypes = [C.POINTER(Problem), _dp, _dp, _dp, _dp]
        L.orc_cholmod.argtypes = [C.c_int, _dp, _dp]
        for f in ("orc_levmar", "orc_trust_region"):
            getattr(L, f).argtypes = [C.POINTER(Problem), _dp, _dp, C.POINTER(Opts), _ip,
                                      C.POINTER(Result)]
        L.orc_solve_hybrid.argtypes = [C.POINTER(Problem), _dp, _dp, C.POINTER(Opts),
                                       C.POINTER(Result)]
        L.orc_pair_count.argtypes = [C.POINTER(Problem)]
        L.orc_pair_count.restype = C.c_longlong
        L.orc_session_new.argtypes = [C.POINTER(Problem)]
        L.orc_session_new.restype = C.c_void_p
        for f in ("orc_session_levmar", "orc_session_trust_region"):
            getattr(L, f).argtypes = [C.c_void_p, _dp, _dp, C.POINTER(Opts), _ip, C.POINTER(Result)]
        L.orc_session_free.argtypes = [C.c_void_p]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def whitening(cov):
    """Per observation (a, b, c) of the upper factor L = [[a, b], [0, c]]
    with L^T L = cov^-1, for (O, 2, 2) covariances."""
    cov = np.asarray(cov, dtype=np.float64).reshape(-1, 2, 2)
    det = cov[:, 0, 0] * cov[:, 1, 1] - cov[:, 0, 1] * cov[:, 1, 0]
    p, q, r = cov[:, 1, 1] / det, -cov[:, 0, 1] / det, cov[:, 0, 0] / det
    a = np.sqrt(p)
    b = q / a
    return np.ascontiguousarray(np.stack([a, b, np.sqrt(r - b * b)], axis=1))


class OracleProblem:
    """Keeps the scene arrays alive for the C problem struct."""

    def __init__(self, scene):
        self.K = _f64(scene.K)
        self.q0 = _f64(scene.q0)
        self.meas = _f64(scene.meas)
        self.obs_pt = np.ascontiguousarray(scene.obs_pt, dtype=np.int32)
        self.obs_cam = np.ascontiguousarray(scene.obs_cam, dtype=np.int32)
        self.nc, self.np_, self.no = scene.n_cams, scene.n_pts, scene.n_obs
        self.cnp = int(getattr(scene, "cnp", 6))
        cov = getattr(scene, "cov", None)
        self.wt = None if cov is None else whitening(cov)
        self.c = Problem(self.nc, self.np_, self.no, _d(self.K), _d(self.q0), _d(self.meas),
                         _i(self.obs_pt), _i(self.obs_cam), self.cnp,
                         None if self.wt is None else _d(self.wt))

    @property
    def ref(self):
        return C.byref(self.c)


def default_opts(**kw):
    o = Opts()
    lib().orc_default_opts(C.byref(o))
    names = {f[0] for f in Opts._fields_}
    for k, v in kw.items():
        if k not in names:
            raise KeyError(k)
        setattr(o, k, v)
    return o


# ---------------------------------------------------------------- stages

def residual(pr, cams, pts):
    ex = np.empty(2 * pr.no)
    lib().orc_residual(pr.ref, _d(_f64(cams)), _d(_f64(pts)), _d(ex))
    return ex.reshape(-1, 2)


def sumsq(x):
    x = _f64(x).ravel()
    return lib().orc_sumsq(x.size, _d(x))


def jacobian(pr, cams, pts):
    JA = np.empty((pr.no, 2, pr.cnp))
    JB = np.empty((pr.no, 2, 3))
    lib().orc_jacobian(pr.ref, _d(_f64(cams)), _d(_f64(pts)), _d(JA), _d(JB))
    return JA, JB


def normal_blocks(pr, JA, JB, ex, coeff=1.0):
    c = pr.cnp
    U = np.empty((pr.nc, c, c))
    V = np.empty((pr.np_, 3, 3))
    W = np.empty((pr.no, c, 3))
    g = np.empty(c * pr.nc + 3 * pr.np_)
    d = np.empty(c * pr.nc + 3 * pr.np_)
    lib().orc_normal_blocks(pr.ref, _d(_f64(JA)), _d(_f64(JB)), _d(_f64(ex)), float(coeff), _d(U),
                            _d(V), _d(W), _d(g), _d(d))
    return U, V, W, g, d


def vinv(V, mu):
    V = _f64(V)
    out = np.empty_like(V)
    lib().orc_vinv(V.shape[0], _d(V), float(mu), _d(out))
    return out


def yblocks(pr, W, Vinv):
    Y = np.empty((pr.no, pr.cnp, 3))
    lib().orc_yblocks(pr.ref, _d(_f64(W)), _d(_f64(Vinv)), _d(Y))
    return Y


def schur(pr, U, mu, Y, W):
    N = pr.cnp * pr.nc
    S = np.zeros((N, N))
    lib().orc_schur(pr.ref, _d(_f64(U)), float(mu), _d(_f64(Y)), _d(_f64(W)), _d(S))
    return np.tril(S)


def ea(pr, Y, g):
    out = np.empty(pr.cnp * pr.nc)
    lib().orc_ea(pr.ref, _d(_f64(Y)), _d(_f64(g)), _d(out))
    return out


def spd_inverse(S):
    S = np.array(S, dtype=np.float64, order="C")
    st = lib().orc_spd_inverse(S.shape[0], _d(S))
    return st, S


def cholesky(S):
    S = np.array(S, dtype=np.float64, order="C")
    st = lib().orc_cholesky(S.shape[0], _d(S))
    return st, S


def chol_solve(L, b):
    L = _f64(L)
    b = _f64(b)
    x = np.empty_like(b)
    lib().orc_chol_solve(L.shape[0], _d(L), _d(b), _d(x))
    return x


def matvec(M, v):
    M = _f64(M)
    out = np.empty(M.shape[0])
    lib().orc_matvec(M.shape[0], _d(M), _d(_f64(v)), _d(out))
    return out


def eb_dpb(pr, W, Vinv, g, dpa):
    eb = np.empty(3 * pr.np_)
    dpb = np.empty(3 * pr.np_)
    lib().orc_eb_dpb(pr.ref, _d(_f64(W)), _d(_f64(Vinv)), _d(_f64(g)), _d(_f64(dpa)), _d(eb), _d(dpb))
    return eb, dpb


def jmultiply(pr, JA, JB, x):
    out = np.empty(2 * pr.no)
    lib().orc_jmultiply(pr.ref, _d(_f64(JA)), _d(_f64(JB)), _d(_f64(x)), _d(out))
    return out


def cholmod(S):
    S = np.array(S, dtype=np.float64, order="C")
    E = np.empty(S.shape[0])
    lib().orc_cholmod(S.shape[0], _d(S), _d(E))
    return S, E


# ---------------------------------------------------------------- drivers

class Run:
    def __init__(self, status, iterations, initial_cost, final_cost, trace, cams, pts):
        self.status = status
        self.iterations = iterations
        self.initial_cost = initial_cost
        self.final_cost = final_cost
        self.trace = trace
        self.cams = cams
        self.pts = pts


def _drive(fn, scene, opts, itno0=0, trace_cap=4096):
    pr = OracleProblem(scene)
    cams = _f64(scene.cams).copy()
    pts = _f64(scene.pts).copy()
    tr = np.zeros(trace_cap, dtype=TRACE_DTYPE)
    res = Result(0, 0, 0.0, 0.0, 0, trace_cap, tr.ctypes.data_as(C.POINTER(Trace)))
    if fn == "hybrid":
        lib().orc_solve_hybrid(pr.ref, _d(cams), _d(pts), C.byref(opts), C.byref(res))
    else:
        it = C.c_int(itno0)
        getattr(lib(), fn)(pr.ref, _d(cams), _d(pts), C.byref(opts), C.byref(it), C.byref(res))
    n = min(res.n_trace, trace_cap)
    return Run(res.status, res.iterations, res.initial_cost, res.final_cost, tr[:n].copy(), cams, pts)


def levmar(scene, opts=None, **kw):
    return _drive("orc_levmar", scene, opts or default_opts(**kw))


def trust_region(scene, opts=None, **kw):
    return _drive("orc_trust_region", scene, opts or default_opts(**kw))


def solve_hybrid(scene, opts=None, **kw):
    return _drive("hybrid", scene, opts or default_opts(**kw))


def pair_count(scene):
    pr = OracleProblem(scene)
    return lib().orc_pair_count(pr.ref)


class Session:
    """Oracle problem with index lists built once (for timing repeated LM calls)."""

    def __init__(self, scene):
        self.pr = OracleProblem(scene)
        self.cams0 = _f64(scene.cams).copy()
        self.pts0 = _f64(scene.pts).copy()
        self.s = lib().orc_session_new(self.pr.ref)
        if not self.s:
            raise MemoryError("oracle session")

    def levmar(self, opts, cams=None, pts=None, itno=0, trace_cap=256):
        cams = self.cams0.copy() if cams is None else _f64(cams).copy()
        pts = self.pts0.copy() if pts is None else _f64(pts).copy()
        tr = np.zeros(trace_cap, dtype=TRACE_DTYPE)
        res = Result(0, 0, 0.0, 0.0, 0, trace_cap, tr.ctypes.data_as(C.POINTER(Trace)))
        it = C.c_int(itno)
        lib().orc_session_levmar(self.s, _d(cams), _d(pts), C.byref(opts), C.byref(it), C.byref(res))
        n = min(res.n_trace, trace_cap)
        return Run(res.status, res.iterations, res.initial_cost, res.final_cost, tr[:n].copy(), cams, pts)

    def close(self):
        if self.s:
            lib().orc_session_free(self.s)
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

"""psba_gb300 — sparse bundle adjustment on one GB300 (sm_103a).

Python mirror of the reference's solver interface over the C ABI in
``include/psba.h``: ``levmar`` (PSBA/levmar.h), ``trust_region``
(PSBA/trust_region.h) and the LM/TR alternation of PSBA/main.cpp
(``solve_hybrid``), with the reference's status codes and constants.

The compute runs in ``libpsba_gb300.so`` (hand-written CUDA for sm_103a);
there is no CPU fallback: importing works anywhere, but creating a solver
raises if the library is missing or no CUDA device is present.
"""
import ctypes as C
import os

import numpy as np

from . import scenes  # noqa: F401  (seeded synthetic scenes)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libpsba_gb300.so")

# status codes (PSBA/psba.h:12-18)
ITER_TURN_TO_LM, ITER_TURN_TO_TR, ITER_CONTINUE, ITER_ERR = 1, 2, 3, 4
ITER_DP_NO_CHANGE, ITER_ERR_SMALL_ENOUGH, ITER_PASS = 5, 6, 7
STATUS_NAMES = {1: "TURN_TO_LM", 2: "TURN_TO_TR", 3: "CONTINUE", 4: "ERR", 5: "DP_NO_CHANGE",
                6: "ERR_SMALL_ENOUGH", 7: "PASS"}
TRACE_LM_TRIAL, TRACE_LM_SOLVE_FAIL, TRACE_TR_TRIAL, TRACE_TR_PB_FAIL, TRACE_LM_STOP = 1, 2, 3, 4, 5
PREC_FP64, PREC_MIXED = 0, 1

PSBA_OK, PSBA_ERR_ARG, PSBA_ERR_CUDA, PSBA_ERR_NOMEM, PSBA_ERR_STATE = 0, -1, -2, -3, -4

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class ProblemDesc(C.Structure):
    _fields_ = [("n_cams", C.c_int), ("n_pts", C.c_int), ("n_obs", C.c_int), ("K", _dp), ("q0", _dp),
                ("cams", _dp), ("pts", _dp), ("meas", _dp), ("obs_pt", _ip), ("obs_cam", _ip),
                ("cnp", C.c_int), ("cov", _dp)]


class Opts(C.Structure):
    _fields_ = [("tau", C.c_double), ("stop_thresh", C.c_double), ("eps", C.c_double),
                ("eps2", C.c_double), ("max_iter", C.c_int), ("allow_switch", C.c_int),
                ("precision", C.c_int), ("refine", C.c_int)]


class TraceEntry(C.Structure):
    _fields_ = [("itno", C.c_int), ("kind", C.c_int), ("accepted", C.c_int), ("pad", C.c_int),
                ("damping", C.c_double), ("rho", C.c_double), ("cost", C.c_double),
                ("lambda_", C.c_double)]


class Result(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("initial_cost", C.c_double),
                ("final_cost", C.c_double), ("n_trace", C.c_int), ("trace_cap", C.c_int),
                ("trace", C.POINTER(TraceEntry)), ("device_ms", C.c_double), ("n_trials", C.c_int),
                ("n_linearizations", C.c_int)]


TRACE_DTYPE = np.dtype([("itno", np.int32), ("kind", np.int32), ("accepted", np.int32),
                        ("pad", np.int32), ("damping", np.float64), ("rho", np.float64),
                        ("cost", np.float64), ("lambda_", np.float64)])

# every entry point declared in include/psba.h
EXPORTS = ("psba_default_opts", "psba_create", "psba_destroy", "psba_get_params", "psba_set_params",
           "psba_reset_params", "psba_set_precision", "psba_set_refine", "psba_set_wait_limit",
           "psba_levmar", "psba_levmar_resume", "psba_trust_region", "psba_solve_hybrid", "psba_eval_residual",
           "psba_eval_jacobian", "psba_eval_normal", "psba_eval_reduced", "psba_eval_step",
           "psba_eval_jmultiply", "psba_eval_cholmod", "psba_eval_dense_solve", "psba_eval_pivot_reciprocal",
           "psba_last_error", "psba_stream",
           "psba_device_bytes", "psba_version", "psba_set_stage_timing", "psba_set_stage_mask", "psba_get_stage_timing",
           "psba_transfer_bytes", "psba_kernel_launches", "psba_measure_peak", "psba_cost_noalloc",
           "psba_batch_create", "psba_batch_destroy", "psba_batch_levmar", "psba_batch_get_params",
           "psba_batch_reset_params", "psba_batch_set_threads", "psba_batch_set_lanes_per_pair",
           "psba_batch_device_bytes", "psba_server_default_opts", "psba_server_create", "psba_batch_submit",
           "psba_batch_poll", "psba_server_stats_get", "psba_server_destroy")
STAGES = ("linearize", "point_blocks", "camera_blocks", "vinv", "yblocks", "schur_off", "schur_diag",
          "schur_reduce", "cholesky", "eb_dpb", "trial_cost")

_lib = None


class PSBAError(RuntimeError):
    pass


def build():
    """Compile the CUDA library (nvcc, sm_103a)."""
    from . import nvcc_build
    return nvcc_build.build()


def lib():
    """Load libpsba_gb300.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise PSBAError("libpsba_gb300.so is missing: run psba_gb300.build() (nvcc, sm_103a)")
        L = C.CDLL(LIB_PATH)
        L.psba_default_opts.argtypes = [C.POINTER(Opts)]
        L.psba_create.argtypes = [C.POINTER(ProblemDesc), C.POINTER(C.c_void_p)]
        L.psba_destroy.argtypes = [C.c_void_p]
        L.psba_get_params.argtypes = [C.c_void_p, _dp, _dp]
        L.psba_set_params.argtypes = [C.c_void_p, _dp, _dp]
        L.psba_reset_params.argtypes = [C.c_void_p]
        L.psba_set_precision.argtypes = [C.c_void_p, C.c_int]
        L.psba_set_refine.argtypes = [C.c_void_p, C.c_int]
        L.psba_set_wait_limit.argtypes = [C.c_void_p, C.c_longlong]
        for f in ("psba_levmar", "psba_trust_region"):
            getattr(L, f).argtypes = [C.c_void_p, C.POINTER(Opts), _ip, C.POINTER(Result)]
        L.psba_solve_hybrid.argtypes = [C.c_void_p, C.POINTER(Opts), C.POINTER(Result)]
        L.psba_levmar_resume.argtypes = [C.c_void_p, C.POINTER(Opts), C.c_double, C.c_int, C.c_double, _ip,
                                         C.POINTER(Result)]
        L.psba_eval_residual.argtypes = [C.c_void_p, _dp, _dp]
        L.psba_eval_jacobian.argtypes = [C.c_void_p, _dp, _dp]
        L.psba_eval_normal.argtypes = [C.c_void_p, C.c_double, _dp, _dp, _dp, _dp]
        L.psba_eval_reduced.argtypes = [C.c_void_p, C.c_double, _dp, _dp, _dp, _dp]
        L.psba_eval_step.argtypes = [C.c_void_p, _dp, _ip]
        L.psba_eval_jmultiply.argtypes = [C.c_void_p, _dp, _dp]
        L.psba_eval_cholmod.argtypes = [C.c_int, _dp, _dp]
        L.psba_eval_dense_solve.argtypes = [C.c_int, _dp, _dp, _dp, _ip]
        L.psba_eval_pivot_reciprocal.argtypes = [C.c_int, _dp, _dp]
        L.psba_last_error.restype = C.c_char_p
        L.psba_stream.argtypes = [C.c_void_p]
        L.psba_stream.restype = C.c_void_p
        L.psba_device_bytes.argtypes = [C.c_void_p]
        L.psba_device_bytes.restype = C.c_size_t
        L.psba_version.restype = C.c_char_p
        L.psba_set_stage_timing.argtypes = [C.c_void_p, C.c_int]
        L.psba_set_stage_mask.argtypes = [C.c_void_p, C.c_uint]
        L.psba_get_stage_timing.argtypes = [C.c_void_p, _dp, C.POINTER(C.c_longlong), C.c_int]
        L.psba_transfer_bytes.argtypes = [C.c_void_p, C.POINTER(C.c_size_t), C.POINTER(C.c_size_t)]
        L.psba_kernel_launches.restype = C.c_longlong
        L.psba_measure_peak.argtypes = [C.c_int, _dp]
        _lib = L
    return _lib


def _check(rc):
    if rc != PSBA_OK:
        raise PSBAError("psba error %d: %s" % (rc, lib().psba_last_error().decode()))


def _d(a):
    return a.ctypes.data_as(_dp)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def default_opts(**kw):
    o = Opts()
    lib().psba_default_opts(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise KeyError(k)
        setattr(o, k, v)
    return o


class SolveResult:
    def __init__(self, res, trace, cams, pts):
        self.status = res.status
        self.status_name = STATUS_NAMES.get(res.status, str(res.status))
        self.iterations = res.iterations
        self.initial_cost = res.initial_cost
        self.final_cost = res.final_cost
        self.device_ms = res.device_ms
        self.n_trials = res.n_trials
        self.n_linearizations = res.n_linearizations
        self.trace = trace
        self.cams = cams
        self.pts = pts

    def __repr__(self):
        return ("SolveResult(status=%s, iterations=%d, initial_cost=%.6g, final_cost=%.6g, "
                "trials=%d, device_ms=%.3f)" % (self.status_name, self.iterations, self.initial_cost,
                                                self.final_cost, self.n_trials, self.device_ms))


class Solver:
    """One problem resident on the device (the reference's PSBA_struct)."""

    def __init__(self, scene):
        L = lib()
        self.nc, self.np_, self.no = scene.n_cams, scene.n_pts, scene.n_obs
        self.cnp = int(getattr(scene, "cnp", 6))
        self._keep = [_f64(scene.K), _f64(scene.q0), _f64(scene.cams), _f64(scene.pts), _f64(scene.meas),
                      np.ascontiguousarray(scene.obs_pt, dtype=np.int32),
                      np.ascontiguousarray(scene.obs_cam, dtype=np.int32)]
        K, q0, cams, pts, meas, opt, ocam = self._keep
        cov = getattr(scene, "cov", None)
        cov = None if cov is None else _f64(cov).reshape(-1, 2, 2)
        self._keep.append(cov)
        desc = ProblemDesc(self.nc, self.np_, self.no, _d(K), _d(q0), _d(cams), _d(pts), _d(meas),
                           opt.ctypes.data_as(_ip), ocam.ctypes.data_as(_ip), self.cnp,
                           None if cov is None else _d(cov))
        h = C.c_void_p()
        _check(L.psba_create(C.byref(desc), C.byref(h)))
        self.h = h
        self._keep = None

    def close(self):
        if getattr(self, "h", None):
            lib().psba_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def N(self):
        return self.cnp * self.nc

    @property
    def n_params(self):
        return self.cnp * self.nc + 3 * self.np_

    def device_bytes(self):
        return lib().psba_device_bytes(self.h)

    def transfer_bytes(self):
        a, b = C.c_size_t(), C.c_size_t()
        _check(lib().psba_transfer_bytes(self.h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_stage_timing(self, enable=True, stages=None):
        """Stage timing with CUDA events: every stage, or only the named
        ones (names from STAGES); clears the totals."""
        if stages is None:
            _check(lib().psba_set_stage_timing(self.h, 1 if enable else 0))
            return
        mask = 0
        for name in stages:
            mask |= 1 << STAGES.index(name)
        _check(lib().psba_set_stage_mask(self.h, mask if enable else 0))

    def stage_timing(self):
        ms = np.zeros(len(STAGES))
        cnt = np.zeros(len(STAGES), dtype=np.int64)
        n = lib().psba_get_stage_timing(self.h, _d(ms), cnt.ctypes.data_as(C.POINTER(C.c_longlong)), len(STAGES))
        if n < 0:
            _check(n)
        return {STAGES[k]: (float(ms[k]), int(cnt[k])) for k in range(len(STAGES))}

    def stream(self):
        return lib().psba_stream(self.h)

    def get_params(self):
        cams = np.empty((self.nc, self.cnp))
        pts = np.empty((self.np_, 3))
        _check(lib().psba_get_params(self.h, _d(cams), _d(pts)))
        return cams, pts

    def set_params(self, cams, pts):
        _check(lib().psba_set_params(self.h, _d(_f64(cams)), _d(_f64(pts))))

    def set_precision(self, precision):
        """Precision of the eval_* stages: PREC_FP64 or PREC_MIXED."""
        _check(lib().psba_set_precision(self.h, int(precision)))

    def set_refine(self, refine):
        """1: one step of iterative refinement after each reduced solve of the
        eval_* stages (the solves take it from their options)."""
        _check(lib().psba_set_refine(self.h, int(refine)))

    def set_wait_limit(self, polls=0):
        """Polls per device-side wait before it reports a stall (0: default)."""
        _check(lib().psba_set_wait_limit(self.h, int(polls)))

    def reset_params(self):
        """Back to the initial estimate given at creation (device-side copy)."""
        _check(lib().psba_reset_params(self.h))

    def _run(self, fn, opts, itno, trace_cap, fetch):
        tr = np.zeros(max(trace_cap, 1), dtype=TRACE_DTYPE)
        res = Result()
        res.trace_cap = trace_cap
        res.trace = tr.ctypes.data_as(C.POINTER(TraceEntry)) if trace_cap else None
        if fn == "hybrid":
            _check(lib().psba_solve_hybrid(self.h, C.byref(opts), C.byref(res)))
        else:
            it = C.c_int(itno)
            _check(getattr(lib(), fn)(self.h, C.byref(opts), C.byref(it), C.byref(res)))
        n = min(res.n_trace, trace_cap)
        cams, pts = self.get_params() if fetch else (None, None)
        return SolveResult(res, tr[:n].copy(), cams, pts)

    def levmar(self, opts=None, itno=0, trace_cap=4096, fetch=True, **kw):
        return self._run("psba_levmar", opts or default_opts(**kw), itno, trace_cap, fetch)

    def levmar_resume(self, opts, mu, nu, p_L2, itno=0, trace_cap=4096, fetch=True):
        """levmar() continued from an LM state (mu, nu, |p|^2) at the current
        parameters, e.g. a batch problem its iteration cap stopped."""
        tr = np.zeros(max(trace_cap, 1), dtype=TRACE_DTYPE)
        res = Result()
        res.trace_cap = trace_cap
        res.trace = tr.ctypes.data_as(C.POINTER(TraceEntry)) if trace_cap else None
        it = C.c_int(itno)
        _check(lib().psba_levmar_resume(self.h, C.byref(opts), float(mu), int(nu), float(p_L2), C.byref(it),
                                        C.byref(res)))
        n = min(res.n_trace, trace_cap)
        cams, pts = self.get_params() if fetch else (None, None)
        return SolveResult(res, tr[:n].copy(), cams, pts)

    def trust_region(self, opts=None, itno=0, trace_cap=4096, fetch=True, **kw):
        return self._run("psba_trust_region", opts or default_opts(**kw), itno, trace_cap, fetch)

    def solve_hybrid(self, opts=None, trace_cap=4096, fetch=True, **kw):
        return self._run("hybrid", opts or default_opts(**kw), 0, trace_cap, fetch)

    # ---- stage evaluation in the reference's layouts
    def eval_residual(self):
        ex = np.empty((self.no, 2))
        cost = C.c_double()
        _check(lib().psba_eval_residual(self.h, _d(ex), C.byref(cost)))
        return ex, cost.value

    def eval_jacobian(self):
        JA = np.empty((self.no, 2, self.cnp))
        JB = np.empty((self.no, 2, 3))
        _check(lib().psba_eval_jacobian(self.h, _d(JA), _d(JB)))
        return JA, JB

    def eval_normal(self, coeff=1.0):
        U = np.empty((self.nc, self.cnp, self.cnp))
        V = np.empty((self.np_, 3, 3))
        W = np.empty((self.no, self.cnp, 3))
        g = np.empty(self.n_params)
        _check(lib().psba_eval_normal(self.h, float(coeff), _d(U), _d(V), _d(W), _d(g)))
        return U, V, W, g

    def eval_reduced(self, mu):
        Vinv = np.empty((self.np_, 3, 3))
        Y = np.empty((self.no, self.cnp, 3))
        S = np.empty((self.N, self.N))
        ea = np.empty(self.N)
        _check(lib().psba_eval_reduced(self.h, float(mu), _d(Vinv), _d(Y), _d(S), _d(ea)))
        return Vinv, Y, S, ea

    def eval_step(self):
        dp = np.full(self.n_params, np.nan)
        st = C.c_int()
        _check(lib().psba_eval_step(self.h, _d(dp), C.byref(st)))
        return st.value, dp

    def eval_jmultiply(self, x):
        out = np.empty(2 * self.no)
        _check(lib().psba_eval_jmultiply(self.h, _d(_f64(x)), _d(out)))
        return out


def cholmod(S):
    """Modified Cholesky (trust-region lambda fallback) on the device."""
    S = np.array(S, dtype=np.float64, order="C")
    E = np.empty(S.shape[0])
    _check(lib().psba_eval_cholmod(S.shape[0], _d(S), _d(E)))
    return S, E


def dense_solve(S, b):
    """The solver's dense reduced-camera solve on the device: (status, x)
    with x = S^-1 b (S's lower triangle read); status 0 factored, 1 a pivot
    not positive/finite/normal, 2 a device-side wait ran out."""
    S = np.ascontiguousarray(S, dtype=np.float64)
    n = S.shape[0]
    b = _f64(b)
    x = np.full(n, np.nan)
    st = C.c_int(-1)
    _check(lib().psba_eval_dense_solve(n, _d(S), _d(b), _d(x), C.byref(st)))
    return st.value, x


def pivot_reciprocal(x):
    """The dense factor's pivot reciprocal, evaluated on the device."""
    x = _f64(x).ravel()
    y = np.empty_like(x)
    _check(lib().psba_eval_pivot_reciprocal(x.size, _d(x), _d(y)))
    return y


def version():
    return lib().psba_version().decode()


def kernel_launches():
    return int(lib().psba_kernel_launches())


PEAK_KINDS = {"fp64": 0, "fp32": 1, "dmma_m8n8k4": 2, "dmma_m16n8k16": 3, "dmma_and_fp64": 4}


def measure_peak(which="fp64"):
    """Measured throughput in TFLOP/s of the current device: "fp64" / "fp32"
    FMA chains, or the FP64 tensor cores ("dmma_m8n8k4", "dmma_m16n8k16")."""
    t = C.c_double()
    _check(lib().psba_measure_peak(PEAK_KINDS[which], C.byref(t)))
    return t.value

"""Serving: continuous batching of bundle-adjustment requests on one GPU.

``Server`` wraps psba_server_* / psba_batch_submit / psba_batch_poll of
include/psba.h.  Requests are admitted by HBM footprint into a pool owned by
the server, keep their LM state on the device, and advance together a time
slice of LM iterations per persistent launch; new arrivals join the next
launch.  Each request runs the reference's levmar() control flow
(PSBA/levmar.cpp:45-256) and its result does not depend on the mix.

``run_poisson`` drives a server with Poisson arrivals (one submitting thread,
one polling thread; ctypes releases the GIL during the calls) and returns
per-request latencies, for the serving benchmark and tests.
"""
import ctypes as C
import threading
import time

import numpy as np

from . import PREC_FP64, PSBAError, ProblemDesc, _check, _d, _f64, _ip, default_opts, lib, Opts

PSBA_PENDING = 1
PSBA_REQUEST_FAILED = 2  # psba_batch_poll: the request ended with an error


class ServerOpts(C.Structure):
    _fields_ = [("hbm_budget_bytes", C.c_double), ("max_active", C.c_int), ("slice_iters", C.c_int),
                ("threads", C.c_int), ("lanes_per_pair", C.c_int), ("large_cams", C.c_int),
                ("large_lanes", C.c_int), ("large_share", C.c_double), ("large_obs", C.c_int),
                ("fp64_intrinsics", C.c_int), ("large_chol_ctas", C.c_int), ("large_wait_limit", C.c_longlong)]


class RequestResult(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("n_trials", C.c_int),
                ("n_linearizations", C.c_int), ("initial_cost", C.c_double), ("final_cost", C.c_double),
                ("queued_ms", C.c_double), ("latency_ms", C.c_double), ("device_bytes", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("admitted", C.c_longlong), ("finished", C.c_longlong),
                ("launches", C.c_longlong), ("active", C.c_int), ("queued", C.c_int),
                ("bytes_in_use", C.c_double), ("peak_bytes", C.c_double), ("busy_ms", C.c_double)]


_bound = False


def _bind():
    global _bound
    L = lib()
    if not _bound:
        L.psba_server_default_opts.argtypes = [C.POINTER(ServerOpts)]
        L.psba_server_default_opts.restype = None
        L.psba_server_create.argtypes = [C.POINTER(ServerOpts), C.POINTER(Opts), C.POINTER(C.c_void_p)]
        L.psba_batch_submit.argtypes = [C.c_void_p, C.POINTER(ProblemDesc), C.POINTER(C.c_longlong)]
        L.psba_batch_poll.argtypes = [C.c_void_p, C.c_longlong, C.c_int, C.POINTER(RequestResult), C.c_void_p,
                                      C.c_void_p]
        L.psba_server_stats_get.argtypes = [C.c_void_p, C.POINTER(ServerStats)]
        L.psba_server_destroy.argtypes = [C.c_void_p]
        _bound = True
    return L


class Request:
    """A finished request: the solver's result, host-clock timings, parameters."""

    def __init__(self, r, cams, pts, error=None):
        self.error = error  # None, or the message of a request that ended with an error (status: its code)
        self.status = r.status
        self.iterations = r.iterations
        self.n_trials = r.n_trials
        self.initial_cost = r.initial_cost
        self.final_cost = r.final_cost
        self.queued_ms = r.queued_ms
        self.latency_ms = r.latency_ms
        self.device_bytes = r.device_bytes
        self.cams = cams
        self.pts = pts


class Server:
    def __init__(self, precision=PREC_FP64, max_iter=15, hbm_budget_bytes=120e9, max_active=1024,
                 slice_iters=1, threads=256, lanes_per_pair=32, large_cams=None, large_lanes=None,
                 large_share=None, large_obs=None, fp64_intrinsics=None, large_wait_limit=None,
                 large_chol_ctas=None, **lm):
        L = _bind()
        so = ServerOpts()
        L.psba_server_default_opts(C.byref(so))
        so.hbm_budget_bytes = float(hbm_budget_bytes)
        so.max_active = int(max_active)
        so.slice_iters = int(slice_iters)
        so.threads = int(threads)
        so.lanes_per_pair = int(lanes_per_pair)
        if large_cams is not None:
            so.large_cams = int(large_cams)
        if large_lanes is not None:
            so.large_lanes = int(large_lanes)
        if large_share is not None:
            so.large_share = float(large_share)
        if large_obs is not None:
            so.large_obs = int(large_obs)
        if fp64_intrinsics is not None:
            so.fp64_intrinsics = int(bool(fp64_intrinsics))
        if large_wait_limit is not None:
            so.large_wait_limit = int(large_wait_limit)
        if large_chol_ctas is not None:
            so.large_chol_ctas = int(large_chol_ctas)
        o = default_opts(precision=precision, max_iter=max_iter, allow_switch=0, **lm)
        h = C.c_void_p()
        _check(L.psba_server_create(C.byref(so), C.byref(o), C.byref(h)))
        self.h = h
        self._shapes = {}
        self._lock = threading.Lock()

    def submit(self, sc):
        cnp = int(getattr(sc, "cnp", 6))
        cov = getattr(sc, "cov", None)
        arrs = [_f64(sc.K), _f64(sc.q0), _f64(sc.cams), _f64(sc.pts), _f64(sc.meas),
                np.ascontiguousarray(sc.obs_pt, dtype=np.int32), np.ascontiguousarray(sc.obs_cam, dtype=np.int32),
                None if cov is None else _f64(cov).reshape(-1, 2, 2)]
        K, q0, cams, pts, meas, opt, ocam, cv = arrs
        desc = ProblemDesc(sc.n_cams, sc.n_pts, sc.n_obs, _d(K), _d(q0), _d(cams), _d(pts), _d(meas),
                           opt.ctypes.data_as(_ip), ocam.ctypes.data_as(_ip), cnp, None if cv is None else _d(cv))
        t = C.c_longlong()
        _check(lib().psba_batch_submit(self.h, C.byref(desc), C.byref(t)))
        with self._lock:
            self._shapes[t.value] = (sc.n_cams, sc.n_pts, cnp)
        return t.value

    def poll(self, ticket, timeout_ms=0):
        """The finished Request, or None if it is still running."""
        with self._lock:
            nc, npts, cnp = self._shapes[ticket]
        cams = np.empty((nc, cnp))
        pts = np.empty((npts, 3))
        r = RequestResult()
        rc = lib().psba_batch_poll(self.h, ticket, int(timeout_ms), C.byref(r), cams.ctypes.data,
                                   pts.ctypes.data)
        if rc == PSBA_PENDING:
            return None
        if rc == PSBA_REQUEST_FAILED:  # this request alone; the server goes on
            with self._lock:
                del self._shapes[ticket]
            return Request(r, None, None, error=lib().psba_last_error().decode())
        _check(rc)
        with self._lock:
            del self._shapes[ticket]
        return Request(r, cams, pts)

    def wait(self, ticket, timeout_s=600.0):
        t_end = time.time() + timeout_s
        while True:
            r = self.poll(ticket, 200)
            if r is not None:
                return r
            if time.time() > t_end:
                raise PSBAError("request %d did not finish in %.0f s" % (ticket, timeout_s))

    def stats(self):
        st = ServerStats()
        _check(lib().psba_server_stats_get(self.h, C.byref(st)))
        return {f: getattr(st, f) for f, _ in ServerStats._fields_}

    def close(self):
        if self.h:
            lib().psba_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def run_poisson(server, scenes_list, rate, n_requests, seed=0, timeout_s=600.0):
    """Submit n_requests (cycling through scenes_list) at Poisson arrivals of
    `rate` per second; return (per-request dicts, wall seconds from the first
    submission to the last result)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate, size=n_requests)
    tickets = [None] * n_requests
    submitted = threading.Event()
    errors = []

    def submitter():
        t0 = time.perf_counter()
        due = 0.0
        try:
            for q in range(n_requests):
                due += gaps[q]
                delay = t0 + due - time.perf_counter()
                if delay > 0:
                    time.sleep(delay)
                tickets[q] = server.submit(scenes_list[q % len(scenes_list)])
        except Exception as e:  # surfaced by the caller
            errors.append(e)
        finally:
            submitted.set()

    t_start = time.perf_counter()
    th = threading.Thread(target=submitter)
    th.start()
    out = [None] * n_requests
    pending = set(range(n_requests))
    t_end = time.time() + timeout_s
    while pending and not errors:
        if time.time() > t_end:
            raise PSBAError("serving run timed out with %d requests open" % len(pending))
        progressed = False
        for q in sorted(pending):
            if tickets[q] is None:
                continue
            r = server.poll(tickets[q], 0)
            if r is not None:
                out[q] = r
                pending.discard(q)
                progressed = True
        if not progressed:
            time.sleep(0.0005)
    th.join()
    if errors:
        raise errors[0]
    wall = time.perf_counter() - t_start
    return out, wall

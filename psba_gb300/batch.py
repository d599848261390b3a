"""Batches of independent problems (one persistent launch) and its autotuner.

``Batch`` wraps psba_batch_* of include/psba.h: every problem runs the
reference's levmar() control flow (PSBA/levmar.cpp:45-256) inside one CTA of
a persistent kernel.  ``autotune`` picks the tile/segment shape per size
bucket -- lanes per camera pair in the Schur stage for each bucket of
problems (bucketed by the mean number of common points per camera pair), and
threads per CTA for the batch -- by timing one LM iteration of the batch for
each candidate (coordinate descent, best of two runs).
"""
import ctypes as C
import time

import numpy as np

from . import (Opts, PSBAError, ProblemDesc, PREC_FP64, PREC_MIXED, _check, _d, _f64, _ip, default_opts, lib)


class BatchResult(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("n_trials", C.c_int),
                ("n_linearizations", C.c_int), ("initial_cost", C.c_double), ("final_cost", C.c_double),
                ("mu", C.c_double), ("p_L2", C.c_double), ("nu", C.c_int), ("pad", C.c_int)]


RESULT_DTYPE = np.dtype([("status", np.int32), ("iterations", np.int32), ("n_trials", np.int32),
                         ("n_linearizations", np.int32), ("initial_cost", np.float64),
                         ("final_cost", np.float64), ("mu", np.float64), ("p_L2", np.float64),
                         ("nu", np.int32), ("pad", np.int32)])

_bound = False


def _bind():
    global _bound
    L = lib()
    if not _bound:
        L.psba_batch_create.argtypes = [C.POINTER(ProblemDesc), C.c_int, C.POINTER(C.c_void_p)]
        L.psba_batch_destroy.argtypes = [C.c_void_p]
        L.psba_batch_levmar.argtypes = [C.c_void_p, C.POINTER(Opts), C.c_void_p, C.POINTER(C.c_double)]
        L.psba_batch_get_params.argtypes = [C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]
        L.psba_batch_reset_params.argtypes = [C.c_void_p]
        L.psba_batch_set_threads.argtypes = [C.c_void_p, C.c_int]
        L.psba_batch_set_lanes_per_pair.argtypes = [C.c_void_p, C.c_void_p]
        L.psba_batch_device_bytes.argtypes = [C.c_void_p]
        L.psba_batch_device_bytes.restype = C.c_size_t
        _bound = True
    return L


def pair_stats(scene):
    """Mean number of common points per camera pair (drives the Schur shape)."""
    opt = np.asarray(scene.obs_pt, dtype=np.int64)
    cam = np.asarray(scene.obs_cam, dtype=np.int64)
    k = np.bincount(opt, minlength=scene.n_pts)
    entries = int((k * (k - 1) // 2).sum())
    keys = []
    for d in range(1, int(k.max(initial=1))):
        same = opt[d:] == opt[:-d]
        keys.append(cam[d:][same] * scene.n_cams + cam[:-d][same])
    n_pairs = len(np.unique(np.concatenate(keys))) if keys else 0
    return entries / max(n_pairs, 1)


class Batch:
    def __init__(self, scenes_list):
        L = _bind()
        self.n = len(scenes_list)
        self.scenes = scenes_list
        keep, descs = [], (ProblemDesc * self.n)()
        for q, sc in enumerate(scenes_list):
            arrs = [_f64(sc.K), _f64(sc.q0), _f64(sc.cams), _f64(sc.pts), _f64(sc.meas),
                    np.ascontiguousarray(sc.obs_pt, dtype=np.int32), np.ascontiguousarray(sc.obs_cam, dtype=np.int32)]
            keep.append(arrs)
            K, q0, cams, pts, meas, opt, ocam = arrs
            descs[q] = ProblemDesc(sc.n_cams, sc.n_pts, sc.n_obs, _d(K), _d(q0), _d(cams), _d(pts), _d(meas),
                                   opt.ctypes.data_as(_ip), ocam.ctypes.data_as(_ip))
        h = C.c_void_p()
        _check(L.psba_batch_create(descs, self.n, C.byref(h)))
        self.h = h
        self.threads = 256
        self.lanes = np.full(self.n, 32, dtype=np.int32)

    def close(self):
        if getattr(self, "h", None):
            lib().psba_batch_destroy(self.h)
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

    def device_bytes(self):
        return lib().psba_batch_device_bytes(self.h)

    def set_threads(self, t):
        _check(lib().psba_batch_set_threads(self.h, int(t)))
        self.threads = int(t)

    def set_lanes(self, lanes):
        lanes = np.ascontiguousarray(lanes, dtype=np.int32)
        _check(lib().psba_batch_set_lanes_per_pair(self.h, lanes.ctypes.data))
        self.lanes = lanes.copy()

    def reset(self):
        _check(lib().psba_batch_reset_params(self.h))

    def levmar(self, opts=None, **kw):
        o = opts or default_opts(**kw)
        res = np.zeros(self.n, dtype=RESULT_DTYPE)
        ms = C.c_double()
        _check(lib().psba_batch_levmar(self.h, C.byref(o), res.ctypes.data, C.byref(ms)))
        return res, ms.value

    def get_params(self, q):
        sc = self.scenes[q]
        cams = np.empty((sc.n_cams, 6))
        pts = np.empty((sc.n_pts, 3))
        _check(lib().psba_batch_get_params(self.h, int(q), cams.ctypes.data, pts.ctypes.data))
        return cams, pts


def levmar_with_handoff(batch, opts, cap, workers=8):
    """The batch solved to opts.max_iter, with the problems the persistent
    launch has not finished after `cap` iterations handed over to the
    single-problem solver (all SMs per problem, one host thread and stream
    each, up to `workers` at once).  A problem runs LM in one CTA of the
    batched launch, so one that needs many iterations holds the whole launch
    while the other SMs idle; the single-problem solver continues it from
    the batch's parameters and LM state (psba_levmar_resume).  Returns the
    results (the batch's, with the continued problems' replaced), the batch's
    device ms and the hand-over's host ms (handle creation included)."""
    import concurrent.futures as cf
    from . import ITER_CONTINUE, Solver
    o1 = Opts.from_buffer_copy(opts)
    o1.max_iter = min(int(cap), int(opts.max_iter))
    res, batch_ms = batch.levmar(o1)
    todo = [int(q) for q in np.nonzero((res["status"] == ITER_CONTINUE) & (res["iterations"] < opts.max_iter))[0]]

    def one(q):
        cams, pts = batch.get_params(q)
        with Solver(batch.scenes[q]) as s:
            s.set_params(cams, pts)
            r = s.levmar_resume(opts, float(res["mu"][q]), int(res["nu"][q]), float(res["p_L2"][q]),
                                itno=int(res["iterations"][q]), fetch=False, trace_cap=0)
        return q, r

    t0 = time.perf_counter()
    with cf.ThreadPoolExecutor(max_workers=max(1, workers)) as ex:
        done = list(ex.map(one, todo))
    hand_ms = 1e3 * (time.perf_counter() - t0) if todo else 0.0
    out = res.copy()
    for q, r in done:
        out["status"][q] = r.status
        out["iterations"][q] = r.iterations
        out["n_trials"][q] += r.n_trials
        out["n_linearizations"][q] += r.n_linearizations
        out["final_cost"][q] = r.final_cost
    return out, batch_ms, hand_ms, todo


def autotune(batch, precision=PREC_MIXED, n_buckets=3, lane_options=(8, 16, 32), thread_options=(128, 256, 512),
             iters=1, repeats=2):
    """Pick lanes per camera pair for each size bucket and threads per CTA.

    Buckets: quantiles of the mean common points per camera pair.  Each
    candidate is timed on one LM iteration of the whole batch (best of
    `repeats`).  Returns the choice and the timing table."""
    stats = np.array([pair_stats(sc) for sc in batch.scenes])
    edges = np.quantile(stats, np.linspace(0, 1, n_buckets + 1)[1:-1]) if n_buckets > 1 else []
    bucket = np.searchsorted(edges, stats, side="right")
    opts = default_opts(allow_switch=0, max_iter=iters, precision=precision)

    def timed():
        best = None
        for _ in range(repeats):
            batch.reset()
            _, ms = batch.levmar(opts)
            best = ms if best is None else min(best, ms)
        batch.reset()
        return best

    table = []
    lanes = np.full(batch.n, 32, dtype=np.int32)
    batch.set_lanes(lanes)
    for b in range(n_buckets):
        best_l, best_t = None, None
        for l in lane_options:
            trial = lanes.copy()
            trial[bucket == b] = l
            batch.set_lanes(trial)
            t = timed()
            table.append({"bucket": int(b), "lanes": int(l), "threads": batch.threads, "ms": t})
            if best_t is None or t < best_t:
                best_l, best_t = l, t
        lanes[bucket == b] = best_l
        batch.set_lanes(lanes)
    best_th, best_t = batch.threads, None
    for th in thread_options:
        batch.set_threads(th)
        t = timed()
        table.append({"bucket": -1, "lanes": -1, "threads": int(th), "ms": t})
        if best_t is None or t < best_t:
            best_th, best_t = th, t
    batch.set_threads(best_th)
    choice = {"threads": int(best_th),
              "lanes_per_bucket": {int(b): int(lanes[bucket == b][0]) if np.any(bucket == b) else None
                                   for b in range(n_buckets)},
              "bucket_edges_mean_common_points": [float(e) for e in edges]}
    return choice, table


def main(argv=None):
    """``python -m psba_gb300.batch --problems 64 --iters 15``: the bench's
    batch workload (seeded scenes: 5-30 cameras, 200-3,000 points, 3-8 views
    per point) in one batch, solved once untimed and once timed in each form
    (mixed, then FP64); prints solves/s and the launch's device time.  It is
    the command the batched kernel's ncu summary is captured under."""
    import argparse

    from . import scenes
    ap = argparse.ArgumentParser(description="batched LM solves of seeded small problems")
    ap.add_argument("--problems", type=int, default=64)
    ap.add_argument("--iters", type=int, default=15, help="LM iteration cap of every problem")
    ap.add_argument("--seed", type=int, default=1000)
    a = ap.parse_args(argv)
    probs = scenes.batch_scenes(a.problems, seed=a.seed)
    with Batch(probs) as b:
        for tag, prec in (("mixed", PREC_MIXED), ("fp64", PREC_FP64)):
            o = default_opts(allow_switch=0, max_iter=a.iters, precision=prec)
            b.reset()
            b.levmar(o)
            b.reset()
            res, ms = b.levmar(o)
            print("%s: %d problems, %.3f ms, %.1f solves/s, median final cost %.6e"
                  % (tag, b.n, ms, b.n / ms * 1e3, float(np.median(res["final_cost"]))))


if __name__ == "__main__":
    main()

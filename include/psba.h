/*
 * psba_gb300 — sparse bundle adjustment (Levenberg-Marquardt and trust-region
 * dogleg) on one NVIDIA GB300 GPU.  C ABI.
 *
 * This is the drop-in boundary for the reference's solver path.  The
 * reference (shenyan0712/PSBA) exposes its solver as two C++ driver calls
 * over a pre-staged OpenCL buffer set:
 *
 *   int levmar(PSBA_structPtr, int cnp, int pnp, int mnp, int n3Dpts, int nCams,
 *              int n2Dprojs, dtype *finalErr);                         PSBA/levmar.h:6-10
 *   int trust_region(PSBA_structPtr, int cnp, int pnp, int mnp, int n3Dpts,
 *                    int nCams, int n2Dprojs, int *blk_idx, dtype *finalErr);
 *                                                                      PSBA/trust_region.h:5-11
 * with the buffers filled by fill_initBuffer2 / fill_idxBuffer
 * (PSBA/cl_psba.cpp:138-207) and the LM<->TR alternation of PSBA/main.cpp:193-208.
 * Here the buffer set is an opaque handle created from host arrays, and the
 * drivers take an options struct instead of compile-time constants
 * (PSBA/psba.h:3-18).  Everything is plain C: pointers, sizes, status codes.
 * No call exits the process; errors are returned and described by
 * psba_last_error().
 *
 * Parameter layout (the reference's, PSBA/main.cpp:131-149):
 *   K     5 per camera: fx, cx, cy, aspect ratio, skew (held fixed)
 *   q0    4 per camera: initial rotation quaternion s, v1, v2, v3
 *   cams  6 per camera: v1, v2, v3 (vector part of the local rotation
 *         quaternion, composed as q(v) (x) q0) and translation t1, t2, t3
 *   pts   3 per point
 *   meas  2 per observation; observations sorted by (point, camera),
 *         each (point, camera) pair at most once (PSBA/misc.cpp:189-197)
 *
 * Threading: one handle is used by one host thread at a time; handles are
 * independent.  Each handle owns one CUDA stream and its device memory.
 */
#ifndef PSBA_GB300_H
#define PSBA_GB300_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* return codes */
#define PSBA_OK 0
#define PSBA_ERR_ARG -1      /* invalid argument (sizes, ordering, null pointer) */
#define PSBA_ERR_CUDA -2     /* CUDA runtime error (message in psba_last_error) */
#define PSBA_ERR_NOMEM -3    /* device allocation failed */
#define PSBA_ERR_STATE -4    /* handle in an unusable state */

/* solver status codes, identical to PSBA/psba.h:12-18 */
#define PSBA_ITER_TURN_TO_LM 1
#define PSBA_ITER_TURN_TO_TR 2
#define PSBA_ITER_CONTINUE 3
#define PSBA_ITER_ERR 4
#define PSBA_ITER_DP_NO_CHANGE 5
#define PSBA_ITER_ERR_SMALL_ENOUGH 6
#define PSBA_ITER_PASS 7

/* trace record kinds */
#define PSBA_TRACE_LM_TRIAL 1      /* LM trial that produced a step; rho computed */
#define PSBA_TRACE_LM_SOLVE_FAIL 2 /* LM trial whose reduced camera system was not SPD */
#define PSBA_TRACE_TR_TRIAL 3      /* dogleg trial */
#define PSBA_TRACE_TR_PB_FAIL 4    /* TR Gauss-Newton step failed; lambda raised */
#define PSBA_TRACE_LM_STOP 5       /* LM trial ended by the step-size tests */

/* precision of the per-observation stages */
#define PSBA_PREC_FP64 0  /* every stage in FP64 */
#define PSBA_PREC_MIXED 1 /* Jacobian, residual, W, Y stored in FP32 (the projection itself
                             is evaluated in FP64); V, V^-1, the gradient, the Schur
                             accumulation, Cholesky, damping and gain ratio in FP64 */

typedef struct psba_handle psba_handle;

typedef struct {
    int n_cams;
    int n_pts;
    int n_obs;
    const double *K;    /* 5 * n_cams: fx, cx, cy, aspect, skew; unused (may be NULL) when cnp > 6 */
    const double *q0;   /* 4 * n_cams */
    const double *cams; /* cnp * n_cams */
    const double *pts;  /* 3 * n_pts */
    const double *meas; /* 2 * n_obs */
    const int *obs_pt;  /* n_obs, non-decreasing */
    const int *obs_cam; /* n_obs, increasing within a point */
    /* Parameters per camera.  0 or 6: quaternion vector part and translation,
     * intrinsics fixed from K (the reference's only model, CL_files/PSBA.cl:5).
     * 11: followed by the intrinsics fx, cx, cy, aspect, skew (the sba
     * variable-K camera files, data/7camsvarK.txt).  16: followed further by
     * the distortion k1, k2, p1, p2, k3 (data/54camsvarKD.txt).  The 11- and
     * 16-parameter models have no reference kernels; psba_batch_* takes
     * 6-parameter cameras (the server runs the others on its large lane).
     * With them the trust-region driver's lambda fallback runs its 3x3-block
     * modified Cholesky on S padded to a multiple of 3 by an identity block. */
    int cnp;
    /* Optional (NULL: unweighted): per observation the 2x2 covariance of the
     * image measurement, row-major (4 values, symmetric positive definite),
     * as the reference's reader parses it (PSBA/readparams.cpp:272-282,
     * 380-412) and its solver ignores (PSBA/main.cpp:112-113).  Residuals and
     * Jacobian rows are whitened by the upper Cholesky factor L of the
     * inverse covariance (L^T L = cov^-1), so the cost is sum e^T cov^-1 e.
     * psba_batch_* takes unweighted problems (the server runs weighted ones
     * on its large lane). */
    const double *cov;
} psba_problem_desc;

typedef struct {
    double tau;         /* initial damping factor, PSBA_INIT_MU (psba.h:6), 1e-3 */
    double stop_thresh; /* PSBA_STOP_THRESH (psba.h:7), 1e-12 */
    double eps;         /* PSBA_EPSILON (psba.h:8), 1e-12 */
    double eps2;        /* PSBA_EPSILON2 (psba.h:9), 1e-12 */
    int max_iter;       /* shared iteration budget, 50 (levmar.cpp:100) */
    int allow_switch;   /* 1: LM hands over to TR after 5 good steps (levmar.cpp:215-219) */
    int precision;      /* PSBA_PREC_* */
    int refine;         /* 1: one step of iterative refinement after each reduced solve:
                           r = ea - S dpa against a copy of S, formed as an accurate dot
                           product (twice the working precision), then both triangular solves
                           with the factor, added into dpa; the forward error of dpa falls
                           from ~cond(S) eps to ~eps.  Per-handle solver only (the batched
                           and serving engines refuse it); default 0 */
} psba_opts;

typedef struct {
    int itno;
    int kind;     /* PSBA_TRACE_* */
    int accepted; /* 1 if the parameters were updated */
    int pad;
    double damping; /* mu (LM) or trust radius before the trial (TR) */
    double rho;     /* gain ratio, NaN when not computed */
    double cost;    /* sum of squared residuals at the trial point, NaN when not computed */
    double lambda;  /* TR: lambda of the Gauss-Newton step */
} psba_trace_entry;

typedef struct {
    int status;           /* PSBA_ITER_* of the last driver */
    int iterations;       /* shared iteration counter on return */
    double initial_cost;  /* sum of squared residuals before the first step */
    double final_cost;    /* the driver's finalErr */
    int n_trace;          /* number of trace records produced (may exceed trace_cap) */
    int trace_cap;        /* capacity of trace (caller-set) */
    psba_trace_entry *trace; /* caller-owned buffer of trace_cap records, or NULL */
    double device_ms;     /* GPU time of the solve, CUDA events on the handle's stream */
    int n_trials;         /* damping trials run */
    int n_linearizations; /* Jacobian evaluations run */
} psba_result;

/* ---- lifetime ---------------------------------------------------------- */

/* Default options: the reference's compile-time constants (PSBA/psba.h:3-18). */
void psba_default_opts(psba_opts *opts);

/* Replaces setup_cl + fill_initBuffer2 + generate_idxs + fill_idxBuffer
 * (PSBA/cl_psba.cpp:16-207, PSBA/misc.cpp:178-218): validates the problem,
 * copies it to the device and builds the camera-sorted and camera-pair
 * index lists there.  The host arrays may be freed afterwards. */
int psba_create(const psba_problem_desc *desc, psba_handle **out);

/* Replaces release of the PSBA_struct buffers. */
int psba_destroy(psba_handle *h);

/* Current parameters (the reference updates cams_buffer / pts3D_buffer in
 * place, sba_func.cpp:1170-1214). */
int psba_get_params(psba_handle *h, double *cams, double *pts);
int psba_set_params(psba_handle *h, const double *cams, const double *pts);

/* Restores the initial estimate given to psba_create, on the device (the
 * reference re-reads its input files instead, PSBA/main.cpp:102-180). */
int psba_reset_params(psba_handle *h);

/* ---- drivers ----------------------------------------------------------- */

/* levmar(), PSBA/levmar.cpp:45-256.  *itno is the shared iteration counter
 * (the reference's global itno, main.cpp:27); it is advanced in place. */
int psba_levmar(psba_handle *h, const psba_opts *opts, int *itno, psba_result *res);

/* trust_region(), PSBA/trust_region.cpp:49-288 (dogleg / 2-D subspace step
 * with the modified-Cholesky lambda fallback). */
int psba_trust_region(psba_handle *h, const psba_opts *opts, int *itno, psba_result *res);

/* The LM <-> TR alternation of PSBA/main.cpp:193-208, from itno = 0. */
int psba_solve_hybrid(psba_handle *h, const psba_opts *opts, psba_result *res);

/* levmar() continued from a given LM state (mu, nu, |p|^2 of the current
 * parameters, e.g. a psba_batch_result of a problem its iteration cap
 * stopped) at the handle's current parameters and shared iteration count
 * *itno: the first linearization does not re-initialise mu (levmar.cpp:
 * 114-120 runs only for a fresh solve); otherwise psba_levmar. */
int psba_levmar_resume(psba_handle *h, const psba_opts *opts, double mu, int nu, double p_L2, int *itno,
                       psba_result *res);

/* Bound of the handle's device-side waits: the dense factor's waits on its
 * task flags and the Y kernel's wait for its bulk copies, in polls (0: the
 * default, 2^22, about half a second).  A wait that runs out ends its kernel
 * with a status the driver reads; the solve then returns PSBA_ERR_STATE and
 * the handle stays usable.  No reference counterpart: the reference's
 * device-side enqueue chain has no waits of its own (CL_files/SPD_inv.cl:165-179). */
int psba_set_wait_limit(psba_handle *h, long long polls);

/* ---- stage evaluation (parity checks; reference layouts, host buffers) -- */

/* Precision used by the psba_eval_* calls (PSBA_PREC_*); the drivers take it
 * from their options.  No reference counterpart: the reference is FP64 only
 * (CL_files/PSBA.cl:2). */
int psba_set_precision(psba_handle *h, int precision);

/* Refinement step of the psba_eval_step calls (0 or 1, see psba_opts.refine);
 * the drivers take it from their options.  No reference counterpart: the
 * reference inverts S explicitly (SPD_inv.cl) and multiplies once
 * (matVec_mul, cl_linearalg.cpp:19). */
int psba_set_refine(psba_handle *h, int refine);

/* compute_exQT (sba_func.cpp:81-145): ex = meas - projection; *cost = sum ex^2. */
int psba_eval_residual(psba_handle *h, double *ex, double *cost);

/* compute_jacobiQT (sba_func.cpp:153-245): JA 2x6 and JB 2x3 per observation. */
int psba_eval_jacobian(psba_handle *h, double *JA, double *JB);

/* compute_U/V/Wblks/g (sba_func.cpp:252-617) with factor coeff: U 6x6 per
 * camera, V 3x3 per point, W 6x3 per observation, g = [ga | gb]. */
int psba_eval_normal(psba_handle *h, double coeff, double *U, double *V, double *W, double *g);

/* After psba_eval_normal: one damping trial's reduced system
 * (update_UV, compute_Vinv, compute_Yblks, compute_S, compute_ea;
 * levmar.cpp:126-131): Vinv 3x3 per point, Y 6x3 per observation,
 * S (6C x 6C, lower triangle defined, upper set to zero), ea (6C). */
int psba_eval_reduced(psba_handle *h, double mu, double *Vinv, double *Y, double *S, double *ea);

/* After psba_eval_reduced: the step dp = [dpa | dpb] of SPDinv + matVec_mul +
 * compute_eb + compute_dpb (levmar.cpp:134-155).  *chol_status is 0 when S
 * was factored, 1 when it was not SPD (dp untouched). */
int psba_eval_step(psba_handle *h, double *dp, int *chol_status);

/* compute_Jmultiply (sba_func.cpp:19-75) for the last Jacobian: out holds the
 * 2 entries per observation (the reference's dense grid minus its zeros). */
int psba_eval_jmultiply(psba_handle *h, const double *x, double *out);

/* Modified Cholesky of cholmod_blk + compute_cholmod_E (cl_cholmod.cpp:25-202)
 * on an n x n matrix (lower triangle read); writes the factor (lower) to S
 * and the diagonal correction to E.  Runs on the device; n % 3 == 0. */
int psba_eval_cholmod(int n, double *S, double *E);

/* The reduced-camera solve of psba_eval_step (Cholesky factor with the
 * forward solve carried along, then the back solve) on an n x n matrix given
 * by the caller: S row-major, lower triangle read, 1 <= n <= 4096; x = S^-1 b.
 * *status is 0 when S was factored, 1 when a pivot was not positive, finite
 * and normal (the reference's failure test, SPD_inv.cl:66-107; subnormal
 * pivots count as failures here), 2 when a device-side wait ran out.
 * Replaces SPDinv + matVec_mul (PSBA/cl_spdinv.cpp:18-40,
 * PSBA/cl_linearalg.cpp:19-55) for parity checks at any size. */
int psba_eval_dense_solve(int n, const double *S, const double *b, double *x, int *status);

/* The dense factor's pivot reciprocal (the hardware's approximate reciprocal
 * refined by one order-3 Householder step) applied to n values on the
 * device, for accuracy checks against the correctly rounded 1.0 / x.  No
 * reference counterpart: the reference divides (SPD_inv.cl:60-111). */
int psba_eval_pivot_reciprocal(int n, const double *x, double *y);

/* ---- measurement (no reference counterpart: the reference only keeps
 * host clock() totals, PSBA/main.cpp:22-37,220-227) ---------------------- */

/* Stage timing with CUDA events on the handle's stream.  enable != 0 turns
 * it on and clears the totals.  Stage order: linearize (camera tables,
 * residual, Jacobian, W), point blocks (V, gb), camera blocks (U, ga), V^-1,
 * Y, Schur off-diagonal, Schur diagonal + ea, Schur reduction, Cholesky +
 * solves, eb/dpb, trial cost. */
#define PSBA_N_STAGES 11
int psba_set_stage_timing(psba_handle *h, int enable);
/* Times only the stages whose bit is set (bit k: stage k in the order above)
 * and clears the totals; 0 turns timing off.  Each timed stage costs two
 * events per occurrence on the stream. */
int psba_set_stage_mask(psba_handle *h, unsigned mask);
/* Fills total_ms[k] and counts[k] for k < n; returns the number of stages. */
int psba_get_stage_timing(psba_handle *h, double *total_ms, long long *counts, int n);

/* Host<->device bytes copied by the handle so far (problem upload, index
 * lists, parameter read-back). */
int psba_transfer_bytes(psba_handle *h, size_t *h2d, size_t *d2h);

/* Kernels launched by this library in the process so far. */
long long psba_kernel_launches(void);

/* Throughput of the current device in TFLOP/s: which = 0 FP64 FMA, 1 FP32
 * FMA, 2 FP64 tensor cores (mma.sync m8n8k4), 3 FP64 tensor cores (mma.sync
 * m16n8k16), 4 both FP64 paths at once (half the warps m8n8k4, half FMA,
 * equal flops).  Eight independent chains per thread or warp. */
int psba_measure_peak(int which, double *tflops);

/* ---- batches of independent problems ------------------------------------ */

/* Many independent small problems solved in one persistent launch (a CUDA
 * graph of [queue reset, kernel]): each CTA takes a problem from a device
 * queue and runs levmar() (PSBA/levmar.cpp:45-256) for it with every stage
 * done by the CTA.  A problem's result does not depend on the batch it is in.
 * The reference solves one problem per process; it has no counterpart. */
typedef struct psba_batch psba_batch;
typedef struct {
    int status;      /* PSBA_ITER_* */
    int iterations;
    int n_trials;
    int n_linearizations;
    double initial_cost;
    double final_cost;
    /* LM state at exit (for psba_levmar_resume when the iteration cap ended
     * the solve): damping mu, its growth factor nu, |p|^2 of the last accepted
     * parameters (levmar.cpp:73-249) */
    double mu;
    double p_L2;
    int nu;
    int pad;
} psba_batch_result;

int psba_batch_create(const psba_problem_desc *problems, int n_problems, psba_batch **out);
int psba_batch_destroy(psba_batch *b);
/* Runs LM on every problem (opts->precision selects the form); results has
 * n_problems entries; *device_ms = GPU time of the launch. */
int psba_batch_levmar(psba_batch *b, const psba_opts *opts, psba_batch_result *results, double *device_ms);
int psba_batch_get_params(psba_batch *b, int problem, double *cams, double *pts);
int psba_batch_reset_params(psba_batch *b);
/* Tile/segment shape knobs set by the autotuner (psba_gb300.batch.autotune):
 * threads per CTA (128, 256, 512) and, per problem, lanes per camera pair in
 * the Schur stage (8, 16, 32). */
int psba_batch_set_threads(psba_batch *b, int threads);
int psba_batch_set_lanes_per_pair(psba_batch *b, const int *lanes);
size_t psba_batch_device_bytes(psba_batch *b);

/* ---- serving: continuous batching of solve requests -------------------- */

/* A server owns one HBM pool and a worker thread (the batch lane), plus
 * large_lanes threads (the large lane).  Requests with more than large_cams
 * cameras go to the large lane: each is solved by the single-problem engine
 * (psba_create / psba_levmar: multi-CTA kernels and the dataflow Cholesky
 * over the whole GPU) on its own stream, concurrently with the batch lane;
 * its device memory counts against large_share of the budget.  The rest of
 * the budget is the batch lane's pool.  Requests with more than large_obs
 * observations, 11- or 16-parameter cameras, or covariances also take the
 * large lane.
 * psba_batch_submit lays a request out on the calling thread and queues it;
 * the worker admits queued requests in arrival order while a resident slot is
 * free and the request fits the pool, and advances all resident problems
 * together, a time slice of LM iterations per persistent launch (the
 * heaviest problem runs slice_iters iterations, lighter ones proportionally
 * more).  Parameters, linearisation and LM state stay on the device between
 * slices; a request arriving while others run joins the next launch, and a
 * finished one leaves at the end of its launch and frees its memory.  A
 * request's result is bit-identical alone and in any mix.
 *
 * Reference: none -- the reference solves one problem per process
 * (PSBA/main.cpp:193-208); each request is solved by levmar()
 * (PSBA/levmar.cpp:45-256) with the LM-to-TR hand-over off. */
typedef struct psba_server psba_server;

typedef struct psba_server_opts {
    double hbm_budget_bytes; /* all device memory the server may hold for requests (default 120e9) */
    int max_active;          /* resident problems of the batch lane at once (default 1024) */
    int slice_iters;         /* outer LM iterations of the heaviest problem per launch (default 1) */
    int threads;             /* CTA size of the persistent launch: 128, 256, 512 (default 256) */
    int lanes_per_pair;      /* lanes per camera pair in the Schur stage: 8, 16, 32 (default 32) */
    int large_cams;          /* requests with more cameras run on the large lane (default 40; 0: no large lane) */
    int large_lanes;         /* large-lane host threads, each solving one request at a time (default 8) */
    double large_share;      /* share of hbm_budget_bytes reserved for the large lane (default 0.25) */
    int large_obs;           /* ... and so do requests with more observations (default 20000; 0: no limit) */
    int fp64_intrinsics;     /* 1: requests with 11/16-parameter cameras are solved in FP64 even when the
                                server's precision is mixed (default 1: with FP32 Jacobian columns for the
                                intrinsics, LM converges slowly or stalls short of the FP64 minimum) */
    int large_chol_ctas;     /* CTAs of each large-lane solve's dense factor (default 0: the SMs divided by
                                large_lanes, so the lanes' factors run side by side) */
    long long large_wait_limit; /* polls per device-side wait of a large-lane solve (psba_set_wait_limit;
                                   default 0: the library's); a wait that runs out fails that request
                                   alone (PSBA_REQUEST_FAILED from psba_batch_poll) */
} psba_server_opts;

typedef struct psba_request_result {
    int status; /* PSBA_ITER_* */
    int iterations;
    int n_trials;
    int n_linearizations;
    double initial_cost;
    double final_cost;
    double queued_ms;    /* submit to admission (host clock) */
    double latency_ms;   /* submit to result ready (host clock) */
    double device_bytes; /* pool bytes held while resident */
} psba_request_result;

typedef struct psba_server_stats {
    long long submitted, admitted, finished, launches;
    int active, queued;
    double bytes_in_use, peak_bytes;
    double busy_ms; /* GPU time of all slice launches */
} psba_server_stats;

#define PSBA_PENDING 1        /* psba_batch_poll: not finished yet */
#define PSBA_REQUEST_FAILED 2 /* psba_batch_poll: the request ended with an error (res->status holds it) */

void psba_server_default_opts(psba_server_opts *o);
/* lm: tau, thresholds, max_iter and precision for every request. */
int psba_server_create(const psba_server_opts *so, const psba_opts *lm, psba_server **out);
/* Never waits for the GPU.  PSBA_ERR_NOMEM if the problem alone exceeds the
 * budget, PSBA_ERR_ARG if it is malformed. */
int psba_batch_submit(psba_server *s, const psba_problem_desc *desc, long long *ticket);
/* PSBA_OK: finished; *res, and cams (6 per camera) / pts (3 per point) when
 * not NULL, are written and the ticket is released.  PSBA_PENDING: not
 * finished within timeout_ms (0: return at once).  PSBA_REQUEST_FAILED: the
 * request alone ended with an error (e.g. PSBA_ERR_STATE: a large-lane dense
 * factor's device wait ran out while other work held the SMs); res->status
 * holds that error code, psba_last_error() the message, the ticket is
 * released and the server goes on.  PSBA_ERR_ARG: unknown ticket.
 * PSBA_ERR_CUDA: the server stopped on a device error. */
int psba_batch_poll(psba_server *s, long long ticket, int timeout_ms, psba_request_result *res, double *cams,
                    double *pts);
int psba_server_stats_get(psba_server *s, psba_server_stats *st);
/* Stops after the launch in flight; unfinished requests are dropped. */
int psba_server_destroy(psba_server *s);

/* ---- cost evaluation without device allocation ------------------------ */

/* Sum of squared reprojection residuals of an unweighted problem with
 * 6-parameter cameras and fixed K (for such a problem, what
 * psba_eval_residual returns in *cost; it takes no covariances and no 11/16-
 * parameter cameras), for callers that cannot allocate device memory when
 * they need it: code running while a CUDA stream is being captured into a
 * graph (cudaMalloc is not allowed then), a serving loop held to a fixed HBM
 * budget, or a host framework that owns all device memory.  No counterpart
 * in the reference.
 *
 * Every pointer is a device pointer the caller owns, in this header's layout
 * (K 5, q0 4, cams 6 per camera; pts 3 per point; meas 2 per observation;
 * obs_pt, obs_cam per observation); *cost (device) receives the result on
 * `stream` (a cudaStream_t, NULL for the default stream).  The indices are
 * checked on the device: an observation whose point index is outside
 * 0..n_pts-1 or camera index outside 0..n_cams-1 is skipped and makes *cost
 * NaN.  Nothing is allocated: the scratch (camera tables and block sums) is a
 * fixed 1 MiB array inside the library, held by every GPU that loads it until
 * the process exits.  Limits: n_cams <= 1024, n_obs <= 16,777,216; larger
 * sizes return PSBA_ERR_ARG.  The first call on a device looks up the array's
 * device address (no allocation); make that first call before any stream
 * capture begins.  All calls on a device share the array and keep the last
 * call's contents, so calls that overlap on the GPU race: order them. */
int psba_cost_noalloc(int n_cams, int n_pts, int n_obs, const double *K, const double *q0, const double *cams,
                      const double *pts, const double *meas, const int *obs_pt, const int *obs_cam,
                      double *cost, void *stream);

/* ---- misc -------------------------------------------------------------- */

/* Message of the last error on the calling thread. */
const char *psba_last_error(void);

/* CUDA stream (cudaStream_t) of the handle, for callers that time or order
 * their own work around a solve. */
void *psba_stream(psba_handle *h);

/* Device bytes held by the handle. */
size_t psba_device_bytes(psba_handle *h);

/* Library version string. */
const char *psba_version(void);

#ifdef __cplusplus
}
#endif
#endif

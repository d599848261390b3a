// Host side of the solver: problem set-up, the LM / trust-region / hybrid
// drivers and the C ABI of include/psba.h.
//
// The drivers keep the reference's control flow (PSBA/levmar.cpp:45-256,
// PSBA/trust_region.cpp:49-405,520-595, PSBA/main.cpp:193-208) and its
// constants; all vector and matrix work runs on the device, and each damping
// trial returns its scalars (Cholesky status, |dp|^2, gain-ratio denominator,
// new cost) to the host in one small copy.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <algorithm>
#include <memory>
#include <string>
#include <mutex>
#include <vector>

#include "psba_internal.h"

namespace psba {

static thread_local std::string g_last_error;

const char *set_error(const std::string &msg)
{
    g_last_error = msg;
    return g_last_error.c_str();
}

}  // namespace psba

using namespace psba;

#define PSBA_CUDA_TRY(expr)                                                                    \
    do {                                                                                       \
        cudaError_t _e = (expr);                                                               \
        if (_e != cudaSuccess) {                                                               \
            set_error(std::string("CUDA error: ") + cudaGetErrorString(_e) + " at " #expr);    \
            return PSBA_ERR_CUDA;                                                              \
        }                                                                                      \
    } while (0)

// Stages timed with CUDA events when stage timing is on (psba_set_stage_timing).
enum Stage {
    ST_LINEARIZE = 0,  // camera tables + residual/Jacobian/W
    ST_POINT,          // V, gb
    ST_CAMERA,         // U, ga
    ST_VINV,
    ST_Y,
    ST_SCHUR_OFF,
    ST_SCHUR_DIAG,
    ST_SCHUR_REDUCE,
    ST_CHOL,           // Cholesky + both triangular solves
    ST_EBDPB,          // eb, dpb, step scalars
    ST_COST,           // residual cost at p + dp
    ST_N
};

struct StageTimer {
    cudaEvent_t a = nullptr, b = nullptr;
    bool pending = false;
    double total_ms = 0.0;
    long long count = 0;
};

struct psba_handle {
    DeviceProblem d;
    unsigned timing = 0;  // stages timed with events: bit k for stage k
    StageTimer timers[ST_N];
    size_t h2d_bytes = 0, d2h_bytes = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::vector<void *> allocs;
    double *scratch = nullptr;   // device scalars for reductions (64 doubles)
    int nred = 0;                // blocks of the long-vector reductions
    int linearized = 0;          // 1 after eval_normal / a linearization
    double last_mu = 0.0;
    double *host_scalars = nullptr;  // pinned, 64 doubles
    int chol_epoch = 0;              // increases with every dense-solver launch
    int refine = 0;                  // 1: one refinement step after each reduced solve
};

namespace {

// Device memory comes from the device's stream-ordered pool
// (cudaMallocAsync / cudaFreeAsync on the handle's stream): creating and
// destroying a handle then never synchronises the device, so handles come
// and go (the serving engine's large lane) while other streams run.  The
// pool keeps freed memory for reuse (release threshold raised once per
// device, for this process only).
void keep_pool_memory()
{
    static std::mutex mu;
    static bool done[MAX_DEVICES] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAX_DEVICES) return;
    std::lock_guard<std::mutex> lk(mu);
    if (done[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        unsigned long long thr = ~0ULL;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
    }
    done[dev] = true;
}

// Small pinned host buffers (trial scalars), reused across handles: freeing
// pinned memory can synchronise the device.
std::mutex g_pinned_mu;
std::vector<std::pair<size_t, void *>> g_pinned_free;

void *pinned_get(size_t bytes)
{
    {
        std::lock_guard<std::mutex> lk(g_pinned_mu);
        for (size_t k = 0; k < g_pinned_free.size(); ++k)
            if (g_pinned_free[k].first == bytes) {
                void *p = g_pinned_free[k].second;
                g_pinned_free.erase(g_pinned_free.begin() + (long)k);
                return p;
            }
    }
    void *p = nullptr;
    return cudaMallocHost(&p, bytes) == cudaSuccess ? p : nullptr;
}

void pinned_put(void *p, size_t bytes)
{
    if (!p) return;
    std::lock_guard<std::mutex> lk(g_pinned_mu);
    g_pinned_free.emplace_back(bytes, p);
}

template <typename P>
int dalloc(psba_handle *h, P **ptr, size_t count)
{
    *ptr = nullptr;
    if (count == 0) count = 1;
    void *p = nullptr;
    cudaError_t e = cudaMallocAsync(&p, count * sizeof(P), h->stream);
    if (e != cudaSuccess) {
        set_error(std::string("device allocation failed: ") + cudaGetErrorString(e));
        return PSBA_ERR_NOMEM;
    }
    h->allocs.push_back(p);
    h->d.bytes += count * sizeof(P);
    *ptr = static_cast<P *>(p);
    return PSBA_OK;
}

template <typename P>
int upload(psba_handle *h, P *dst, const P *src, size_t count)
{
    if (count == 0) return PSBA_OK;
    PSBA_CUDA_TRY(cudaMemcpyAsync(dst, src, count * sizeof(P), cudaMemcpyHostToDevice, h->stream));
    h->h2d_bytes += count * sizeof(P);
    return PSBA_OK;
}

#define TRY(x)                  \
    do {                        \
        int _r = (x);           \
        if (_r != PSBA_OK) return _r; \
    } while (0)

int check_launch()
{
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error(std::string("kernel launch failed: ") + cudaGetErrorString(e));
        return PSBA_ERR_CUDA;
    }
    return PSBA_OK;
}

void collect_timers(psba_handle *h)
{
    for (int k = 0; k < ST_N; ++k) {
        StageTimer &t = h->timers[k];
        if (!t.pending) continue;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, t.a, t.b) == cudaSuccess) {
            t.total_ms += ms;
            t.count++;
        }
        t.pending = false;
    }
}

int sync(psba_handle *h)
{
    cudaError_t e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) {
        set_error(std::string("CUDA error: ") + cudaGetErrorString(e));
        return PSBA_ERR_CUDA;
    }
    if (h->timing) collect_timers(h);
    return check_launch();
}

// Brackets the launches of one stage with events when stage timing is on.
struct StageScope {
    psba_handle *h;
    int k;
    StageScope(psba_handle *h_, int k_) : h(h_), k(k_)
    {
        if ((h->timing >> k) & 1u) cudaEventRecord(h->timers[k].a, h->stream);
    }
    ~StageScope()
    {
        if ((h->timing >> k) & 1u) {
            cudaEventRecord(h->timers[k].b, h->stream);
            h->timers[k].pending = true;
        }
    }
};

// ---------------------------------------------------------------------------
// device work units

struct Scalars {
    // read back from h->scratch
    double v[64];
};

// scratch slots (doubles)
enum {
    SC_MAXDIAG = 0,
    SC_COST = 1,
    SC_PL2A = 2,
    SC_PL2B = 3,
    SC_GTG = 4,
    SC_GTBG = 5,
    SC_PUBPU = 6,
    SC_PUBPB = 7,
    SC_PBBPB = 8,
    SC_PUG = 9,
    SC_PBG = 10,
    SC_PNORM = 11,
    SC_PUN = 12,
    SC_PBN = 13,
    SC_DA = 14,
    SC_DB = 15,
    SC_DC = 16,
    SC_JXN = 17,
    SC_GP = 18,
    SC_ESUM = 19,
    SC_TMP = 32,  // workspace for the dogleg sums
};

int read_scalars(psba_handle *h, double *out)
{
    PSBA_CUDA_TRY(cudaMemcpyAsync(h->host_scalars, h->scratch, 64 * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->stream));
    h->d2h_bytes += 64 * sizeof(double);
    TRY(sync(h));
    std::memcpy(out, h->host_scalars, 64 * sizeof(double));
    return PSBA_OK;
}

int read_trial(psba_handle *h, TrialScalars *t)
{
    PSBA_CUDA_TRY(cudaMemcpyAsync(h->d.scal_host, h->d.scal, sizeof(TrialScalars),
                                  cudaMemcpyDeviceToHost, h->stream));
    PSBA_CUDA_TRY(cudaMemcpyAsync(h->host_scalars, h->scratch, 64 * sizeof(double),
                                  cudaMemcpyDeviceToHost, h->stream));
    h->d2h_bytes += sizeof(TrialScalars) + 64 * sizeof(double);
    TRY(sync(h));
    *t = *h->d.scal_host;
    return PSBA_OK;
}

// Residual cost at the current parameters (into scratch[SC_COST]).
void enqueue_cost_current(psba_handle *h, double *ex_out)
{
    DeviceProblem &d = h->d;
    launch_cam_tables(d, d.cams, nullptr, d.camtab, h->stream);
    const int nb = residual_blocks(d);
    launch_residual(d, d.camtab, d.pts, nullptr, ex_out, d.red_partial, nb, h->scratch + SC_COST, h->stream);
}

// Cost at p + step (into scal->new_cost).
#ifndef PSBA_MIXED_DF_COST
#define PSBA_MIXED_DF_COST 1  // the mixed form's LM trial cost in double-float FP32 arithmetic (else FP64)
#endif

void enqueue_cost_trial(psba_handle *h, const double *step)
{
    DeviceProblem &d = h->d;
    StageScope sc(h, ST_COST);
    const int nb = residual_blocks(d);
    // partials after the eb partials region so they do not collide
    double *part = d.red_partial + 2 * eb_blocks(d) + 8;
    // the mixed form's LM trial (its step d.dp, whose trial points k_eb_dpb
    // has just split into FP32 pairs): the double-float cost
    const bool df = PSBA_MIXED_DF_COST && d.prec == PSBA_PREC_MIXED && d.cnp == 6 && !d.wt && step == d.dp &&
                    (size_t)d.nc * RES_TAB2F * sizeof(float2) <= 48 * 1024;
    launch_cam_tables(d, d.cams, step, d.camtab_new, h->stream, nullptr, df ? d.tab2f : nullptr);
    if (df)
        launch_residual_df(d, part, nb, &d.scal->new_cost, h->stream);
    else
        launch_residual(d, d.camtab_new, d.pts, step + d.N, nullptr, part, nb, &d.scal->new_cost, h->stream);
}

// Jacobian, U, V, W, g with factor coeff at the current parameters.
void enqueue_linearize(psba_handle *h, double coeff)
{
    DeviceProblem &d = h->d;
    {
        StageScope sc(h, ST_LINEARIZE);
        launch_cam_tables(d, d.cams, nullptr, d.camtab, h->stream,
                          d.prec == PSBA_PREC_MIXED && d.cnp == 6 ? d.camtab32 : nullptr,
                          linearize_df(d) ? d.tab2f : nullptr, 1);
        launch_linearize(d, coeff, h->stream);
    }
    {
        StageScope sc(h, ST_POINT);
        launch_point_blocks(d, coeff, h->stream);
    }
    {
        StageScope sc(h, ST_CAMERA);
        launch_camera_blocks(d, coeff, h->stream);
    }
}

// Reduced system for damping mu: V^-1, Y, S, ea (rhs).
void enqueue_reduced(psba_handle *h, double mu)
{
    DeviceProblem &d = h->d;
    {
        StageScope sc(h, ST_VINV);
        launch_vinv(d, mu, h->stream);
    }
    {
        StageScope sc(h, ST_Y);
        launch_yblocks(d, h->stream);
    }
    {
        StageScope sc(h, ST_SCHUR_OFF);
        launch_schur_off(d, h->stream);
    }
    {
        StageScope sc(h, ST_SCHUR_DIAG);
        launch_schur_diag(d, h->stream);
    }
    {
        StageScope sc(h, ST_SCHUR_REDUCE);
        launch_schur_reduce(d, mu, h->stream);
    }
}

// Cholesky + solves -> dpa into dp[0..N), then eb, dpb, scalars.
void enqueue_step(psba_handle *h, double mu)
{
    DeviceProblem &d = h->d;
    {
        StageScope sc(h, ST_CHOL);
        if (h->refine) {  // the factor overwrites S and ea: keep copies for the residual
            cudaMemcpy2DAsync(d.Ssave, sizeof(double) * d.Nm3, d.S, sizeof(double) * d.Np, sizeof(double) * d.Np,
                              d.Np, cudaMemcpyDeviceToDevice, h->stream);
            cudaMemcpyAsync(d.rsave, d.rhs, sizeof(double) * d.Np, cudaMemcpyDeviceToDevice, h->stream);
        }
        launch_chol_dataflow(d, ++h->chol_epoch, d.xsol, h->stream);
        if (h->refine) launch_refine(d, d.Ssave, d.Nm3, d.rsave, d.xsol, h->stream);
        cudaMemcpyAsync(d.dp, d.xsol, sizeof(double) * d.N, cudaMemcpyDeviceToDevice, h->stream);
    }
    {
        StageScope sc(h, ST_EBDPB);
        launch_eb_dpb(d, mu, h->stream);
        launch_finish_trial(d, mu, h->stream);
    }
}

void enqueue_param_norm(psba_handle *h)
{
    DeviceProblem &d = h->d;
    launch_param_norm(d, h->nred, d.red_partial + 4, h->scratch + SC_PL2A, h->scratch + SC_PL2B, h->stream);
}

void trace_push(psba_result *res, int itno, int kind, int acc, double damping, double rho, double cost,
                double lambda)
{
    if (!res) return;
    if (res->trace && res->n_trace < res->trace_cap) {
        psba_trace_entry &t = res->trace[res->n_trace];
        t.itno = itno;
        t.kind = kind;
        t.accepted = acc;
        t.pad = 0;
        t.damping = damping;
        t.rho = rho;
        t.cost = cost;
        t.lambda = lambda;
    }
    res->n_trace++;
}

// ---------------------------------------------------------------------------
// levmar(), PSBA/levmar.cpp:45-256

// An LM state to continue from (psba_levmar_resume).
struct LmState {
    double mu, p_L2;
    int nu;
};

int levmar_impl(psba_handle *h, const psba_opts *o, int *itno, psba_result *res, int *flag_out,
                const LmState *from = nullptr)
{
    DeviceProblem &d = h->d;
    const double tau = o->tau;
    double mu = 0.0, p_L2 = 0.0, ex_L2 = 0.0;
    int nu = 2, gooditer_cnt = 0;
    bool first = true;
    double sc[64];
    if (from) {
        mu = from->mu;
        p_L2 = from->p_L2;
        nu = from->nu;
        first = false;
    }

    enqueue_cost_current(h, nullptr);
    TRY(check_launch());
    TRY(read_scalars(h, sc));
    ex_L2 = sc[SC_COST];
    if (res) res->initial_cost = ex_L2;

    int iter_flag = PSBA_ITER_CONTINUE;
    bool have_pl2_pending = false;
    for (; *itno < o->max_iter && iter_flag == PSBA_ITER_CONTINUE; (*itno)++) {
        enqueue_linearize(h, 1.0);
        if (res) res->n_linearizations++;
        h->linearized = 1;
        if (first) {
            launch_max_uvdiag(d, h->scratch + SC_MAXDIAG, h->stream);
            TRY(check_launch());
            TRY(read_scalars(h, sc));
            mu = tau * sc[SC_MAXDIAG];
            first = false;
            p_L2 = 1e+3;
            nu = 2;
        }
        while (true) {
            enqueue_reduced(h, mu);
            enqueue_step(h, mu);
            enqueue_cost_trial(h, d.dp);
            TRY(check_launch());
            TrialScalars ts;
            TRY(read_trial(h, &ts));
            if (ts.chol_status == 2)
                return set_error("dense solver wait budget exhausted (device dataflow stalled)"), PSBA_ERR_STATE;
            if (res) res->n_trials++;
            if (have_pl2_pending) {
                p_L2 = h->host_scalars[SC_PL2A] + h->host_scalars[SC_PL2B];
                have_pl2_pending = false;
            }
            if (ts.chol_status == 0) {
                const double dp_L2 = ts.dp_L2;
                if (dp_L2 < p_L2 * o->stop_thresh * o->stop_thresh) {
                    iter_flag = PSBA_ITER_DP_NO_CHANGE;
                    trace_push(res, *itno, PSBA_TRACE_LM_STOP, 0, mu, NAN, NAN, 0);
                    break;
                }
                if (dp_L2 >= (p_L2 + o->stop_thresh) / (o->eps * o->eps)) {
                    iter_flag = PSBA_ITER_ERR;
                    trace_push(res, *itno, PSBA_TRACE_LM_STOP, 0, mu, NAN, NAN, 0);
                    break;
                }
                const double new_ex_L2 = ts.new_cost;
                const double rho = (ex_L2 - new_ex_L2) / ts.rho_den;
                if (rho > 0) {
                    const double mu_used = mu;
                    double tmp = 2 * rho - 1;
                    tmp = 1.0 - tmp * tmp * tmp;
                    mu = mu * ((tmp >= (1.0 / 3.0)) ? tmp : (1.0 / 3.0));
                    nu = 2;
                    launch_update_params(d, h->stream);
                    enqueue_param_norm(h);
                    TRY(check_launch());
                    have_pl2_pending = true;
                    ex_L2 = new_ex_L2;
                    trace_push(res, *itno, PSBA_TRACE_LM_TRIAL, 1, mu_used, rho, new_ex_L2, 0);
                    if (std::fabs(rho - 1) < (1.0 / 5.0)) {
                        gooditer_cnt++;
                        if (gooditer_cnt >= 5 && o->allow_switch) {
                            iter_flag = PSBA_ITER_TURN_TO_TR;
                            break;
                        }
                    } else {
                        gooditer_cnt = 0;
                    }
                    break;
                }
                trace_push(res, *itno, PSBA_TRACE_LM_TRIAL, 0, mu, rho, new_ex_L2, 0);
            } else {
                gooditer_cnt = 0;
                trace_push(res, *itno, PSBA_TRACE_LM_SOLVE_FAIL, 0, mu, NAN, NAN, 0);
            }
            mu *= nu;
            const int nu2 = (int)(2u * (unsigned)nu);  // the reference's int nu wraps at 2^31
            if (nu2 <= nu) {
                iter_flag = PSBA_ITER_ERR;
                break;
            }
            nu = nu2;
        }
        if (ex_L2 <= o->stop_thresh) iter_flag = PSBA_ITER_ERR_SMALL_ENOUGH;
    }
    TRY(sync(h));
    if (res) {
        res->final_cost = ex_L2;
        res->status = iter_flag;
        res->iterations = *itno;
    }
    *flag_out = iter_flag;
    return PSBA_OK;
}

// ---------------------------------------------------------------------------
// trust_region(), PSBA/trust_region.cpp:49-288

int dev_dot(psba_handle *h, const double *x, const double *y, long long n, int slot)
{
    launch_dot(x, y, n, h->d.red_partial, h->nred, h->scratch + slot, h->stream);
    return check_launch();
}

// compute_PB (trust_region.cpp:292-405).  Returns 1 when P_B was formed.
int compute_pb(psba_handle *h, double *lambda, int *solved)
{
    DeviceProblem &d = h->d;
    const long long nt = d.N + 3LL * d.np;
    enqueue_reduced(h, *lambda);
    if (d.Nm3 == d.Np)
        PSBA_CUDA_TRY(cudaMemcpyAsync(d.Ssave, d.S, sizeof(double) * (size_t)d.Np * d.Np,
                                      cudaMemcpyDeviceToDevice, h->stream));
    else
        PSBA_CUDA_TRY(cudaMemcpy2DAsync(d.Ssave, sizeof(double) * d.Nm3, d.S, sizeof(double) * d.Np,
                                        sizeof(double) * d.Np, d.Np, cudaMemcpyDeviceToDevice, h->stream));
    enqueue_step(h, *lambda);
    TRY(check_launch());
    TrialScalars ts;
    TRY(read_trial(h, &ts));
    if (ts.chol_status == 2)
        return set_error("dense solver wait budget exhausted (device dataflow stalled)"), PSBA_ERR_STATE;
    if (ts.chol_status != 0) {
        if (*lambda == 0.0) {
            // modified Cholesky of the saved S (lower, N x N inside the padded
            // Np; N not a multiple of 3: the 3x3-block form runs on S padded
            // to one with its identity rows, lambda from the first N entries)
            const int n3 = d.N % 3 == 0 ? d.N : d.N + (3 - d.N % 3);
            launch_cholmod(d.Ssave, n3, d.Nm3, d.E, d.red_partial, h->stream, d.chol_grid_cap);
            TRY(check_launch());
            std::vector<double> E(d.N);
            PSBA_CUDA_TRY(cudaMemcpyAsync(E.data(), d.E, sizeof(double) * d.N, cudaMemcpyDeviceToHost,
                                          h->stream));
            TRY(sync(h));
            double sum = 0.0;
            for (int i = 0; i < d.N; ++i) sum += E[i];
            *lambda = std::fabs(sum) / d.N;
        } else {
            *lambda = 2 * (*lambda);
        }
        *solved = 0;
        return PSBA_OK;
    }
    launch_axpby(d.vecPB, d.dp, -1.0, nullptr, 0.0, nt, h->stream);
    TRY(check_launch());
    *solved = 1;
    return PSBA_OK;
}

int trust_region_impl(psba_handle *h, const psba_opts *o, int *itno, psba_result *res, int *flag_out)
{
    DeviceProblem &d = h->d;
    const long long nt = d.N + 3LL * d.np;
    const long long no2 = 2LL * d.no;
    int iter_flag = PSBA_ITER_CONTINUE, notgood_cnt = 0, good_iters = 0, nu = 2;
    double ex_L2, dk = 1, lambda = 0, origin_lambda = 0.0;
    double sc[64];

    enqueue_cost_current(h, nullptr);
    TRY(check_launch());
    TRY(read_scalars(h, sc));
    ex_L2 = sc[SC_COST];
    if (res && res->n_trace == 0) res->initial_cost = ex_L2;
    double final_err = ex_L2;

    for (; *itno < o->max_iter; (*itno)++) {
        // U, V, W with factor 2; g = -2 J^T e (exactly the negation of the factor-2 sums)
        enqueue_linearize(h, 2.0);
        if (res) res->n_linearizations++;
        h->linearized = 1;
        launch_axpby(d.g, d.g, -1.0, nullptr, 0.0, nt, h->stream);
        launch_jmultiply(d, d.g, d.jx1, h->stream);
        TRY(dev_dot(h, d.jx1, d.jx1, no2, SC_GTBG));
        TRY(dev_dot(h, d.g, d.g, nt, SC_GTG));
        TRY(read_scalars(h, sc));
        // P_U = -(g gtg) / gtBg with gtBg = 2 |J g|^2 (trust_region.cpp:125-130)
        launch_scale(d.vecPU, d.g, h->scratch + SC_GTG, h->scratch + SC_GTBG, 2.0, -1.0, nt, h->stream);

        int solved = 0;
        while (!solved) {
            const double lam_used = lambda;
            TRY(compute_pb(h, &lambda, &solved));
            if (res) res->n_trials++;
            if (!solved) {
                trace_push(res, *itno, PSBA_TRACE_TR_PB_FAIL, 0, dk, NAN, NAN, lam_used);
                if (origin_lambda != 0.0) {
                    if (nu > 4) {
                        TRY(sync(h));
                        if (res) {
                            res->final_cost = final_err;
                            res->status = PSBA_ITER_TURN_TO_LM;
                            res->iterations = *itno;
                        }
                        *flag_out = PSBA_ITER_TURN_TO_LM;
                        return PSBA_OK;
                    }
                    lambda = lambda * nu;
                    nu = nu * 2;
                }
            } else {
                nu = 2;
                origin_lambda = lambda;
            }
        }
        launch_jmultiply(d, d.vecPU, d.jx1, h->stream);
        launch_jmultiply(d, d.vecPB, d.jx2, h->stream);
        TRY(dev_dot(h, d.jx1, d.jx1, no2, SC_PUBPU));
        TRY(dev_dot(h, d.jx1, d.jx2, no2, SC_PUBPB));
        TRY(dev_dot(h, d.jx2, d.jx2, no2, SC_PBBPB));
        TRY(dev_dot(h, d.vecPU, d.g, nt, SC_PUG));
        TRY(dev_dot(h, d.vecPB, d.g, nt, SC_PBG));
        TRY(dev_dot(h, d.vecPU, d.vecPU, nt, SC_PUN));
        TRY(dev_dot(h, d.vecPB, d.vecPB, nt, SC_PBN));
        TRY(read_scalars(h, sc));
        const double pUtBpU = 2 * sc[SC_PUBPU], pUtBpB = 2 * sc[SC_PUBPB], pBtBpB = 2 * sc[SC_PBBPB];
        const double pUg = sc[SC_PUG], pBg = sc[SC_PBG];
        const double pU_norm = std::sqrt(sc[SC_PUN]), pB_norm = std::sqrt(sc[SC_PBN]);

        iter_flag = PSBA_ITER_CONTINUE;
        while (iter_flag == PSBA_ITER_CONTINUE) {
            const double dk_used = dk;
            // compute_p_2 (trust_region.cpp:520-595)
            {
                const double a = pUtBpU, b = pUtBpB, c = pBtBpB;
                const double eta1 = (pBg * b) / (-b * b + c * a) - (c * pUg) / (-b * b + c * a);
                const double eta2 = (pUg * b) / (-b * b + c * a) - (pBg * a) / (-b * b + c * a);
                launch_axpby(d.vecP, d.vecPU, eta1, d.vecPB, eta2, nt, h->stream);
                TRY(dev_dot(h, d.vecP, d.vecP, nt, SC_PNORM));
                TRY(read_scalars(h, sc));
                const double p_norm = std::sqrt(sc[SC_PNORM]);
                if (p_norm > dk) {
                    if (pU_norm > dk) {
                        launch_axpby(d.vecP, d.vecPU, dk / pU_norm, nullptr, 0.0, nt, h->stream);
                    } else if (pB_norm <= dk) {
                        PSBA_CUDA_TRY(cudaMemcpyAsync(d.vecP, d.vecPB, sizeof(double) * nt,
                                                      cudaMemcpyDeviceToDevice, h->stream));
                    } else {
                        // dogleg: A = |PB-PU|^2, B = 2 (PB-PU).(2PU-PB), C = |2PU-PB|^2 - dk^2
                        double *dv = d.vecP;  // PB - PU
                        double *ev = d.dp;    // 2 PU - PB
                        launch_axpby(dv, d.vecPB, 1.0, d.vecPU, -1.0, nt, h->stream);
                        launch_axpby(ev, d.vecPU, 2.0, d.vecPB, -1.0, nt, h->stream);
                        TRY(dev_dot(h, dv, dv, nt, SC_DA));
                        TRY(dev_dot(h, dv, ev, nt, SC_DB));
                        TRY(dev_dot(h, ev, ev, nt, SC_DC));
                        TRY(read_scalars(h, sc));
                        const double A = sc[SC_DA];
                        const double B = 2 * sc[SC_DB];
                        const double C = sc[SC_DC] - dk * dk;
                        double b2_4ac = B * B - 4 * A * C;
                        if (std::fabs(b2_4ac) < 1e-12) b2_4ac = 0;
                        const double tau = (-B + std::sqrt(b2_4ac)) / (2 * A);
                        // P = PU + (tau - 1) (PB - PU)
                        launch_axpby(d.vecP, d.vecPU, 1.0, dv, tau - 1, nt, h->stream);
                    }
                }
            }
            enqueue_cost_trial(h, d.vecP);
            TRY(check_launch());
            TrialScalars ts;
            TRY(read_trial(h, &ts));
            if (res) res->n_trials++;
            const double act_ex_L2 = ts.new_cost;
            if (std::fabs((ex_L2 - act_ex_L2) / ex_L2) < o->eps2) {
                iter_flag = PSBA_ITER_DP_NO_CHANGE;
                trace_push(res, *itno, PSBA_TRACE_TR_TRIAL, 0, dk_used, NAN, act_ex_L2, lambda);
                break;
            }
            launch_jmultiply(d, d.vecP, d.jx1, h->stream);
            TRY(dev_dot(h, d.jx1, d.jx1, no2, SC_JXN));
            TRY(dev_dot(h, d.g, d.vecP, nt, SC_GP));
            TRY(read_scalars(h, sc));
            const double Jx_norm = 2 * sc[SC_JXN];
            double pred_ex_L2 = sc[SC_GP];
            pred_ex_L2 += ex_L2 + Jx_norm / 2;
            const double rho = (ex_L2 - act_ex_L2) / (ex_L2 - pred_ex_L2);
            int acc = 0;
            if (rho < (1.0 / 4.0) || act_ex_L2 > ex_L2) {
                dk = dk / 4;
            } else if (rho >= (3.0 / 4.0) && act_ex_L2 < ex_L2) {
                iter_flag = PSBA_ITER_PASS;
                acc = 1;
                dk = std::fmin(2 * dk, 10000);
            } else if (rho >= (1.0 / 4.0) && rho < (3.0 / 4.0) && act_ex_L2 < ex_L2) {
                iter_flag = PSBA_ITER_PASS;
                acc = 1;
            } else if (std::isnan(rho)) {
                trace_push(res, *itno, PSBA_TRACE_TR_TRIAL, 0, dk_used, rho, act_ex_L2, lambda);
                TRY(sync(h));
                if (res) {
                    res->final_cost = ex_L2;
                    res->status = PSBA_ITER_TURN_TO_LM;
                    res->iterations = *itno;
                }
                *flag_out = PSBA_ITER_TURN_TO_LM;
                return PSBA_OK;
            }
            if (acc) {
                final_err = act_ex_L2;
                PSBA_CUDA_TRY(cudaMemcpyAsync(d.dp, d.vecP, sizeof(double) * nt, cudaMemcpyDeviceToDevice,
                                              h->stream));
                launch_update_params(d, h->stream);
            }
            trace_push(res, *itno, PSBA_TRACE_TR_TRIAL, acc, dk_used, rho, act_ex_L2, lambda);
            if (std::fabs((act_ex_L2 - ex_L2) / ex_L2) <= o->eps2) {
                iter_flag = PSBA_ITER_ERR_SMALL_ENOUGH;
                break;
            }
            if (rho < 1.0 / 4) {
                notgood_cnt++;
                if (notgood_cnt >= 5) {
                    iter_flag = PSBA_ITER_TURN_TO_LM;
                    break;
                }
            } else {
                notgood_cnt = 0;
            }
            if (rho > 3.0 / 4 && act_ex_L2 < ex_L2) {
                good_iters++;
                if (good_iters >= 10) {
                    lambda = 0.0;
                    origin_lambda = 0.0;
                    good_iters = 0;
                }
            } else {
                good_iters = 0;
            }
            if (rho > (1.0 / 4) && act_ex_L2 < ex_L2) ex_L2 = act_ex_L2;
        }
        if (iter_flag != PSBA_ITER_PASS) break;
    }
    TRY(sync(h));
    if (res) {
        res->final_cost = final_err;
        res->status = iter_flag;
        res->iterations = *itno;
    }
    *flag_out = iter_flag;
    return PSBA_OK;
}

}  // namespace

namespace psba {
void set_chol_grid_cap(psba_handle *h, int cap)
{
    if (h) h->d.chol_grid_cap = cap;
}
}  // namespace psba

// ===========================================================================
// C ABI

namespace {

int validate(const psba_problem_desc *p)
{
    if (!p) return set_error("null problem"), PSBA_ERR_ARG;
    if (p->n_cams <= 0 || p->n_pts < 0 || p->n_obs < 0)
        return set_error("problem sizes must be n_cams > 0, n_pts >= 0, n_obs >= 0"), PSBA_ERR_ARG;
    if (p->cnp != 0 && p->cnp != 6 && p->cnp != 11 && p->cnp != 16)
        return set_error("cnp must be 6, 11 or 16 (0 means 6)"), PSBA_ERR_ARG;
    const bool fixed_k = p->cnp == 0 || p->cnp == 6;
    if ((fixed_k && !p->K) || !p->q0 || !p->cams || (p->n_pts && !p->pts) ||
        (p->n_obs && (!p->meas || !p->obs_pt || !p->obs_cam)))
        return set_error("null array in problem"), PSBA_ERR_ARG;
    if ((long long)p->n_cams * 16 > (1LL << 30) || (long long)p->n_obs * 48 > (1LL << 62))
        return set_error("problem too large"), PSBA_ERR_ARG;
    if (p->cov)
        for (int o = 0; o < p->n_obs; ++o) {
            const double *c = p->cov + 4 * (size_t)o;
            if (!(c[0] > 0) || !(c[3] > 0) || c[1] != c[2] || !(c[0] * c[3] - c[1] * c[2] > 0) ||
                !std::isfinite(c[0] * c[3]))
                return set_error("covariance of observation " + std::to_string(o) +
                                 " is not symmetric positive definite"),
                       PSBA_ERR_ARG;
        }
    for (int o = 0; o < p->n_obs; ++o) {
        const int i = p->obs_pt[o], j = p->obs_cam[o];
        if (i < 0 || i >= p->n_pts || j < 0 || j >= p->n_cams)
            return set_error("observation " + std::to_string(o) + " has an index out of range"),
                   PSBA_ERR_ARG;
        if (o > 0) {
            const int pi = p->obs_pt[o - 1], pj = p->obs_cam[o - 1];
            if (i < pi || (i == pi && j <= pj))
                return set_error("observations must be sorted by (point, camera) without repeats "
                                 "(first violation at " + std::to_string(o) + ")"),
                       PSBA_ERR_ARG;
        }
    }
    return PSBA_OK;
}

int create_impl(const psba_problem_desc *p, psba_handle *h)
{
    DeviceProblem &d = h->d;
    d.nc = p->n_cams;
    d.np = p->n_pts;
    d.no = p->n_obs;
    d.cnp = p->cnp == 0 ? 6 : p->cnp;
    d.N = d.cnp * d.nc;
    d.Np = ((d.N + TILE - 1) / TILE) * TILE;
    const int nc = d.nc, np = d.np, no = d.no;

    // ---- index lists, built on the GPU (replace generate_idxs, misc.cpp:178-218)
    if ((long long)nc * nc > (1LL << 24)) return set_error("more than 4096 cameras is not supported"), PSBA_ERR_ARG;
    if (d.Np > 4096)
        return set_error("reduced camera system larger than 4096 (cameras x parameters per camera)"), PSBA_ERR_ARG;
    TRY(dalloc(h, &d.obs_pt, (size_t)no));
    TRY(dalloc(h, &d.obs_cam, (size_t)no));
    TRY(dalloc(h, &d.pt_start, (size_t)np + 1));
    TRY(dalloc(h, &d.cam_obs, (size_t)no));
    TRY(upload(h, d.obs_pt, p->obs_pt, (size_t)no));
    TRY(upload(h, d.obs_cam, p->obs_cam, (size_t)no));
    // points by observation count, descending (stable): the per-point kernels
    // give a warp points of similar length (views per point follow a power
    // law); each point's own sums keep their order.  Per camera and per
    // chunk of the observation array: observation counts, scanned in (camera,
    // chunk) order into where each chunk's observations of the camera start
    // in cam_obs.
    const int cam_chunk = cam_fill_chunk(nc, no);
    const int n_chunks = no > 0 ? (no + cam_chunk - 1) / cam_chunk : 0;
    std::vector<int> cam_start(nc + 1, 0), chunk_off((size_t)nc * n_chunks, 0);
    {
        std::vector<int> deg(np, 0), order(np > 0 ? np : 1);
        for (int o = 0; o < no; ++o) {
            deg[p->obs_pt[o]]++;
            chunk_off[(size_t)p->obs_cam[o] * n_chunks + o / cam_chunk]++;
        }
        int maxdeg = 0;
        for (int i = 0; i < np; ++i) maxdeg = std::max(maxdeg, deg[i]);
        std::vector<int> start(maxdeg + 2, 0);
        for (int i = 0; i < np; ++i) start[maxdeg - deg[i] + 1]++;
        for (int k = 0; k <= maxdeg; ++k) start[k + 1] += start[k];
        for (int i = 0; i < np; ++i) order[start[maxdeg - deg[i]]++] = i;
        TRY(dalloc(h, &d.pt_order, (size_t)np));
        TRY(upload(h, d.pt_order, order.data(), (size_t)np));
        // eb/dpb warps over the points in this order: m lane triples per
        // point share its observations, so no lane walks more than ~10
        std::vector<int2> ebw;
        for (int s = 0; s < np;) {
            const int m = eb_lanes_per_point(deg[order[s]]);
            ebw.push_back(make_int2(s, m));
            s += std::min(EB_PPW / m, np - s);
        }
        while (ebw.empty() || ebw.size() % EB_WARPS) ebw.push_back(make_int2(np, 1));
        ebw.push_back(make_int2(np, 1));
        d.n_eb_warps = (int)ebw.size() - 1;
        TRY(dalloc(h, &d.eb_warps, ebw.size()));
        TRY(upload(h, d.eb_warps, ebw.data(), ebw.size()));
        int run = 0;
        for (int k = 0; k < nc; ++k) {
            cam_start[k] = run;
            for (int s = 0; s < n_chunks; ++s) {
                const int c = chunk_off[(size_t)k * n_chunks + s];
                chunk_off[(size_t)k * n_chunks + s] = run;
                run += c;
            }
        }
        cam_start[nc] = run;
    }
    // pair-list segments: up to seg_len consecutive observations of one
    // camera's list
    const int seg_len = pair_segment_len(nc, no);
    std::vector<int> seg_cam, seg_first, cam_seg(nc + 1, 0);
    for (int k = 0; k < nc; ++k) {
        for (int b = cam_start[k]; b < cam_start[k + 1]; b += seg_len) {
            seg_cam.push_back(k);
            seg_first.push_back(b);
        }
        cam_seg[k + 1] = (int)seg_cam.size();
    }
    const int nseg = (int)seg_cam.size();
    int *d_cam_start = nullptr, *d_chunk_off = nullptr, *d_seg_cam = nullptr, *d_seg_first = nullptr;
    int *d_seg_cnt = nullptr, *d_off = nullptr;
    TRY(dalloc(h, &d_cam_start, (size_t)nc + 1));
    TRY(dalloc(h, &d_chunk_off, std::max<size_t>(1, chunk_off.size())));
    TRY(dalloc(h, &d_seg_cam, std::max(1, nseg)));
    TRY(dalloc(h, &d_seg_first, std::max(1, nseg)));
    TRY(dalloc(h, &d_seg_cnt, std::max<size_t>(1, (size_t)nseg * nc)));
    TRY(dalloc(h, &d_off, std::max<size_t>(1, (size_t)nseg * nc)));
    TRY(upload(h, d_cam_start, cam_start.data(), (size_t)nc + 1));
    TRY(upload(h, d_chunk_off, chunk_off.data(), chunk_off.size()));
    TRY(upload(h, d_seg_cam, seg_cam.data(), (size_t)nseg));
    TRY(upload(h, d_seg_first, seg_first.data(), (size_t)nseg));
    launch_pt_start(np, no, d.obs_pt, d.pt_start, h->stream);
    launch_cam_fill(nc, no, cam_chunk, d.obs_cam, d_chunk_off, d.cam_obs, h->stream);
    launch_pair_count(nc, nseg, seg_len, d_seg_cam, d_seg_first, d_cam_start, d.cam_obs, d.obs_pt, d.obs_cam,
                      d.pt_start, d_seg_cnt, h->stream);
    std::vector<int> seg_cnt((size_t)nseg * nc), off((size_t)nseg * nc, 0);
    if (!seg_cnt.empty())
        PSBA_CUDA_TRY(cudaMemcpyAsync(seg_cnt.data(), d_seg_cnt, sizeof(int) * seg_cnt.size(),
                                      cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    // camera pairs k > l with common points, numbered in (k, l) order; the
    // entries of pair (k, l) from segment q start at off[q * nc + l]
    std::vector<int> pair_kl;
    std::vector<long long> pair_start(1, 0);
    for (int k = 0; k < nc; ++k)
        for (int l = 0; l < k; ++l) {
            long long c = 0;
            for (int q = cam_seg[k]; q < cam_seg[k + 1]; ++q) c += seg_cnt[(size_t)q * nc + l];
            if (c == 0) continue;
            if (pair_start.back() + c > (1LL << 31) - 1)
                return set_error("too many camera-pair entries"), PSBA_ERR_ARG;
            long long run = pair_start.back();
            for (int q = cam_seg[k]; q < cam_seg[k + 1]; ++q) {
                off[(size_t)q * nc + l] = (int)run;
                run += seg_cnt[(size_t)q * nc + l];
            }
            pair_kl.push_back(k);
            pair_kl.push_back(l);
            pair_start.push_back(run);
        }
    const int n_pairs = (int)pair_kl.size() / 2;
    const long long n_entries = pair_start.back();
    TRY(dalloc(h, &d.pair_kl, 2 * (size_t)n_pairs));
    TRY(dalloc(h, &d.pair_a, (size_t)n_entries));
    TRY(dalloc(h, &d.pair_b, (size_t)n_entries));
    TRY(upload(h, d.pair_kl, pair_kl.data(), pair_kl.size()));
    TRY(upload(h, d_off, off.data(), off.size()));
    launch_pair_fill(nc, nseg, seg_len, d_seg_cam, d_seg_first, d_cam_start, d.cam_obs, d.obs_pt, d.obs_cam,
                     d.pt_start, d_off, d.pair_a, d.pair_b, h->stream);
    TRY(check_launch());
    // Schur work units; execution order longest first
    std::vector<SchurUnit> off_units, off_chunks, diag_units, mx_units;
    std::vector<int> off_start(n_pairs + 1, 0), chunk_start(n_pairs + 1, 0), diag_start(nc + 1, 0),
        mx_start(n_pairs + 1, 0);
    off_units.reserve((size_t)(n_entries / SCHUR_CHUNK) + (size_t)n_pairs);
    for (int q = 0; q < n_pairs; ++q) {
        for (long long b = pair_start[q]; b < pair_start[q + 1]; b += SCHUR_CHUNK) {
            const int cnt = (int)std::min<long long>(SCHUR_CHUNK, pair_start[q + 1] - b);
            off_units.push_back({q, (int)b, cnt, (int)off_units.size()});
        }
        off_start[q + 1] = (int)off_units.size();
    }
    int n_chunk_slots = 0;
    if (d.cnp == 6) {
        // the pair list in equal chunks, one per thread of one resident wave,
        // so every SM gets the same number of products; a chunk writes one
        // slot per pair it touches, slots numbered in list order
        const long long G = std::max(1, schur_off_wave_threads());
        const long long len = std::max<long long>(OFF_MIN_LEN, (n_entries + G - 1) / G);
        off_chunks.reserve((size_t)(n_entries / len) + 1);
        int q = 0;
        for (long long b = 0; b < n_entries; b += len) {
            const long long e = std::min(n_entries, b + len);
            while (pair_start[q + 1] <= b) ++q;
            off_chunks.push_back({q, (int)b, (int)(e - b), n_chunk_slots});
            for (long long sb = b, qq = q;; ++qq) {
                if (sb == pair_start[qq]) chunk_start[qq] = n_chunk_slots;
                ++n_chunk_slots;
                const long long se = std::min(e, pair_start[qq + 1]);
                if (se == e) break;
                sb = se;
            }
        }
        chunk_start[n_pairs] = n_chunk_slots;
        // FP32 products: units of <= MX_UNIT entries of one pair, one warp each
        mx_units.reserve((size_t)(n_entries / MX_UNIT) + (size_t)n_pairs);
        for (int q = 0; q < n_pairs; ++q) {
            for (long long b = pair_start[q]; b < pair_start[q + 1]; b += MX_UNIT) {
                const int cnt = (int)std::min<long long>(MX_UNIT, pair_start[q + 1] - b);
                mx_units.push_back({q, (int)b, cnt, (int)mx_units.size()});
            }
            mx_start[q + 1] = (int)mx_units.size();
        }
    }
    const int dchunk = d.cnp == 6 ? DIAG_SUPER : DIAG_CHUNK;
    for (int j = 0; j < nc; ++j) {
        for (int b = cam_start[j]; b < cam_start[j + 1]; b += dchunk) {
            const int cnt = std::min(dchunk, cam_start[j + 1] - b);
            diag_units.push_back({j, b, cnt, (int)diag_units.size()});
        }
        diag_start[j + 1] = (int)diag_units.size();
    }
    // stable order by count, descending (a counting sort: counts are 1..maxc)
    auto sort_by_count = [](std::vector<SchurUnit> &u, int maxc) {
        std::vector<int> start((size_t)maxc + 2, 0);
        for (const SchurUnit &x : u) start[maxc - x.count + 1]++;
        for (int c = 0; c <= maxc; ++c) start[c + 1] += start[c];
        std::vector<SchurUnit> out(u.size());
        for (const SchurUnit &x : u) out[start[maxc - x.count]++] = x;
        u.swap(out);
    };
    sort_by_count(off_units, SCHUR_CHUNK);
    sort_by_count(mx_units, MX_UNIT);
    sort_by_count(diag_units, dchunk);
    std::vector<CamUnit> cam_units;
    std::vector<int> cam_unit_start(nc + 1, 0);
    for (int j = 0; j < nc; ++j) {
        const int cchunk = d.cnp == 6 ? CAM_SUPER : CAM_CHUNK;
        for (int b = cam_start[j]; b < cam_start[j + 1]; b += cchunk)
            cam_units.push_back({j, b, std::min(cchunk, cam_start[j + 1] - b), 0});
        cam_unit_start[j + 1] = (int)cam_units.size();
    }
    d.n_pairs = n_pairs;
    d.n_pair_entries = n_entries;
    d.n_off_units = (int)off_units.size();
    d.n_off_chunks = (int)off_chunks.size();
    d.n_off_chunk_slots = n_chunk_slots;
    d.n_mx_units = (int)mx_units.size();
    d.n_diag_units = (int)diag_units.size();
    d.n_cam_units = (int)cam_units.size();

    // ---- device memory
    const size_t nt = (size_t)d.N + 3 * (size_t)np;
    TRY(dalloc(h, &d.K, 5 * (size_t)nc));
    TRY(dalloc(h, &d.q0, 4 * (size_t)nc));
    TRY(dalloc(h, &d.meas, 2 * (size_t)no));
    TRY(dalloc(h, &d.meas2f, 2 * (size_t)no));
    TRY(dalloc(h, &d.off_units, off_units.size()));
    TRY(dalloc(h, &d.off_unit_start, (size_t)n_pairs + 1));
    if (d.cnp == 6) {
        TRY(dalloc(h, &d.pair_start, (size_t)n_pairs + 1));
        TRY(dalloc(h, &d.off_chunk_start, (size_t)n_pairs + 1));
        TRY(dalloc(h, &d.off_chunks, off_chunks.size()));
        TRY(dalloc(h, &d.mx_units, mx_units.size()));
        TRY(dalloc(h, &d.mx_unit_start, (size_t)n_pairs + 1));
    }
    TRY(dalloc(h, &d.diag_units, diag_units.size()));
    TRY(dalloc(h, &d.diag_unit_start, (size_t)nc + 1));
    TRY(dalloc(h, &d.cam_units, cam_units.size()));
    TRY(dalloc(h, &d.cam_unit_start, (size_t)nc + 1));
    TRY(dalloc(h, &d.cams, (size_t)d.N));
    TRY(dalloc(h, &d.pts, 3 * (size_t)np));
    TRY(dalloc(h, &d.cams0, (size_t)d.N));
    TRY(dalloc(h, &d.pts0, 3 * (size_t)np));
    TRY(dalloc(h, &d.camtab, (size_t)CAMTAB * nc));
    TRY(dalloc(h, &d.camtab_new, (size_t)CAMTAB * nc));
    TRY(dalloc(h, &d.camtab32, (size_t)CAMTAB32 * nc));
    TRY(dalloc(h, &d.ex, 2 * (size_t)no));
    const size_t cnp = (size_t)d.cnp;
    const size_t cam_nv = d.cnp == 6 ? 27 : varcam_cam_partial(d.cnp);
    const size_t diag_nv = d.cnp == 6 ? 27 : varcam_diag_partial(d.cnp);
    TRY(dalloc(h, &d.A, 2 * cnp * (size_t)no));
    TRY(dalloc(h, &d.B, 6 * (size_t)no));
    TRY(dalloc(h, &d.W, 3 * cnp * (size_t)no));
    TRY(dalloc(h, &d.U, cnp * cnp * (size_t)nc));
    TRY(dalloc(h, &d.V, 6 * (size_t)np));
    TRY(dalloc(h, &d.g, nt));
    TRY(dalloc(h, &d.uvdiag, nt));
    TRY(dalloc(h, &d.cam_partial, cam_nv * cam_units.size()));
    TRY(dalloc(h, &d.Vinv, 6 * (size_t)np));
    TRY(dalloc(h, &d.Vinv2f, 12 * (size_t)np));
    TRY(dalloc(h, &d.gb32, 3 * (size_t)np));
    TRY(dalloc(h, &d.Y, 3 * cnp * (size_t)no));
    TRY(dalloc(h, &d.schur_partial, cnp * cnp * off_partial_slots(d) + diag_nv * diag_units.size()));
    TRY(dalloc(h, &d.S, (size_t)d.Np * d.Np));
    d.Nm3 = d.N % 3 == 0 ? d.Np : ((d.Np + 2) / 3) * 3;
    TRY(dalloc(h, &d.Ssave, (size_t)d.Nm3 * d.Nm3));
    TRY(dalloc(h, &d.rhs, (size_t)d.Np));
    TRY(dalloc(h, &d.rsave, (size_t)d.Np));
    TRY(dalloc(h, &d.dpa2f, (size_t)d.Np));
    TRY(dalloc(h, &d.x2f, 3 * (size_t)np));
    TRY(dalloc(h, &d.tab2f, (size_t)RES_TAB2F * nc));
    TRY(dalloc(h, &d.xsol, (size_t)d.Np));
    TRY(dalloc(h, &d.Linv, (size_t)d.Np * TILE));
    TRY(dalloc(h, &d.status, 4));
    TRY(dalloc(h, &d.tickets, 3));
    {
        const int nb = d.Np / TILE;
        std::vector<int2> tasks;
        chol_task_list(nb, tasks);
        d.chol_n_tasks = (int)tasks.size();
        d.chol_n_flags = nb * (nb + 1) / 2 + 3 * nb;
        TRY(dalloc(h, &d.chol_pre, (size_t)nb * TILE * TILE));
        TRY(dalloc(h, &d.chol_tasks, tasks.size()));
        TRY(dalloc(h, &d.chol_flags, (size_t)d.chol_n_flags));
        TRY(upload(h, d.chol_tasks, tasks.data(), tasks.size()));
        PSBA_CUDA_TRY(cudaMemsetAsync(d.chol_flags, 0, sizeof(int) * d.chol_n_flags, h->stream));
    }
    TRY(dalloc(h, &d.dp, nt));
    TRY(dalloc(h, &d.eb, 3 * (size_t)np));
    h->nred = 512;
    const int res_blocks = residual_blocks(d), ebb = eb_blocks(d);
    d.red_partial_cap = std::max<int>({2 * ebb + 8 + res_blocks, h->nred + 8, (int)cholmod_work(d.Nm3)});
    TRY(dalloc(h, &d.red_partial, (size_t)d.red_partial_cap));
    TRY(dalloc(h, &d.scal, 1));
    TRY(dalloc(h, &h->scratch, 64));
    TRY(dalloc(h, &d.vecPU, nt));
    TRY(dalloc(h, &d.vecPB, nt));
    TRY(dalloc(h, &d.vecP, nt));
    TRY(dalloc(h, &d.jx1, 2 * (size_t)no));
    TRY(dalloc(h, &d.jx2, 2 * (size_t)no));
    TRY(dalloc(h, &d.E, (size_t)d.Nm3));
    if (d.Nm3 > d.Np) {
        // the rows and columns past Np stay an identity block: the fallback's
        // copies of S fill only the leading Np x Np part
        std::vector<double> pad((size_t)d.Nm3 * d.Nm3, 0.0);
        for (int r = d.Np; r < d.Nm3; ++r) pad[(size_t)r * d.Nm3 + r] = 1.0;
        TRY(upload(h, d.Ssave, pad.data(), pad.size()));
    }
    TRY(dalloc(h, &d.tmp9, 9 * (size_t)np));
    d.scal_host = static_cast<TrialScalars *>(pinned_get(sizeof(TrialScalars)));
    h->host_scalars = static_cast<double *>(pinned_get(64 * sizeof(double)));
    if (!d.scal_host || !h->host_scalars) return set_error("pinned host allocation failed"), PSBA_ERR_NOMEM;

    if (d.cnp == 6) TRY(upload(h, d.K, p->K, 5 * (size_t)nc));
    TRY(upload(h, d.q0, p->q0, 4 * (size_t)nc));
    TRY(upload(h, d.meas, p->meas, 2 * (size_t)no));
    launch_split2f(d.meas, d.meas2f, 2LL * no, h->stream);  // the mixed trial cost's measurements
    if (p->cov && no) {
        // whitening L (upper, L^T L = cov^-1) per observation
        std::vector<double> w(3 * (size_t)no);
        for (int o = 0; o < no; ++o) {
            const double *c = p->cov + 4 * (size_t)o;
            const double det = c[0] * c[3] - c[1] * c[2];
            const double pi = c[3] / det, qi = -c[1] / det, ri = c[0] / det;  // cov^-1
            const double a = std::sqrt(pi), b = qi / a;
            w[3 * (size_t)o] = a;
            w[3 * (size_t)o + 1] = b;
            w[3 * (size_t)o + 2] = std::sqrt(ri - b * b);
        }
        TRY(dalloc(h, &d.wt, 3 * (size_t)no));
        TRY(upload(h, d.wt, w.data(), w.size()));
    }
    TRY(upload(h, d.off_units, off_units.data(), off_units.size()));
    TRY(upload(h, d.off_unit_start, off_start.data(), off_start.size()));
    if (d.cnp == 6) {
        const std::vector<int> ps(pair_start.begin(), pair_start.end());
        TRY(upload(h, d.pair_start, ps.data(), ps.size()));
        TRY(upload(h, d.off_chunk_start, chunk_start.data(), chunk_start.size()));
        TRY(upload(h, d.off_chunks, off_chunks.data(), off_chunks.size()));
        TRY(upload(h, d.mx_units, mx_units.data(), mx_units.size()));
        TRY(upload(h, d.mx_unit_start, mx_start.data(), mx_start.size()));
    }
    TRY(upload(h, d.diag_units, diag_units.data(), diag_units.size()));
    TRY(upload(h, d.diag_unit_start, diag_start.data(), diag_start.size()));
    TRY(upload(h, d.cam_units, cam_units.data(), cam_units.size()));
    TRY(upload(h, d.cam_unit_start, cam_unit_start.data(), cam_unit_start.size()));
    TRY(upload(h, d.cams, p->cams, (size_t)d.N));
    TRY(upload(h, d.pts, p->pts, 3 * (size_t)np));
    PSBA_CUDA_TRY(cudaMemcpyAsync(d.cams0, d.cams, sizeof(double) * d.N, cudaMemcpyDeviceToDevice, h->stream));
    PSBA_CUDA_TRY(cudaMemcpyAsync(d.pts0, d.pts, sizeof(double) * 3 * (size_t)np, cudaMemcpyDeviceToDevice,
                                  h->stream));
    PSBA_CUDA_TRY(cudaMemsetAsync(d.status, 0, 4 * sizeof(int), h->stream));
    PSBA_CUDA_TRY(cudaMemsetAsync(d.tickets, 0, 3 * sizeof(int), h->stream));
    PSBA_CUDA_TRY(cudaMemsetAsync(d.scal, 0, sizeof(TrialScalars), h->stream));
    PSBA_CUDA_TRY(cudaMemsetAsync(h->scratch, 0, 64 * sizeof(double), h->stream));
    return sync(h);  // host vectors go out of scope after the copies complete
}

void destroy_impl(psba_handle *h)
{
    if (!h) return;
    if (h->stream) {
        for (void *p : h->allocs) cudaFreeAsync(p, h->stream);
        cudaStreamSynchronize(h->stream);
    }
    pinned_put(h->d.scal_host, sizeof(TrialScalars));
    pinned_put(h->host_scalars, 64 * sizeof(double));
    for (int k = 0; k < ST_N; ++k) {
        if (h->timers[k].a) cudaEventDestroy(h->timers[k].a);
        if (h->timers[k].b) cudaEventDestroy(h->timers[k].b);
    }
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

void reset_result(psba_result *res)
{
    if (!res) return;
    res->status = 0;
    res->iterations = 0;
    res->initial_cost = NAN;
    res->final_cost = NAN;
    res->n_trace = 0;
    res->device_ms = 0.0;
    res->n_trials = 0;
    res->n_linearizations = 0;
}

int timed_begin(psba_handle *h)
{
    PSBA_CUDA_TRY(cudaEventRecord(h->ev0, h->stream));
    return PSBA_OK;
}

int timed_end(psba_handle *h, psba_result *res)
{
    PSBA_CUDA_TRY(cudaEventRecord(h->ev1, h->stream));
    PSBA_CUDA_TRY(cudaEventSynchronize(h->ev1));
    float ms = 0.f;
    PSBA_CUDA_TRY(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    if (res) res->device_ms = ms;
    return PSBA_OK;
}

// Device array of the per-observation / per-point storage type -> host doubles.
int copy_out(psba_handle *h, double *dst, const double *src, size_t count)
{
    if (count == 0 || !dst) return PSBA_OK;
    if (h->d.prec == PSBA_PREC_FP64) {
        PSBA_CUDA_TRY(cudaMemcpyAsync(dst, src, sizeof(double) * count, cudaMemcpyDeviceToHost, h->stream));
        return PSBA_OK;
    }
    std::vector<float> tmp(count);
    PSBA_CUDA_TRY(cudaMemcpyAsync(tmp.data(), src, sizeof(float) * count, cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    for (size_t k = 0; k < count; ++k) dst[k] = tmp[k];
    return PSBA_OK;
}

int check_opts(const psba_opts *o)
{
    if (!o) return set_error("null options"), PSBA_ERR_ARG;
    if (o->precision != PSBA_PREC_FP64 && o->precision != PSBA_PREC_MIXED)
        return set_error("unknown precision"), PSBA_ERR_ARG;
    if (o->refine != 0 && o->refine != 1) return set_error("refine must be 0 or 1"), PSBA_ERR_ARG;
    return PSBA_OK;
}

}  // namespace

extern "C" {

void psba_default_opts(psba_opts *o)
{
    if (!o) return;
    o->tau = 1e-3;
    o->stop_thresh = 1e-12;
    o->eps = 1e-12;
    o->eps2 = 1e-12;
    o->max_iter = 50;
    o->allow_switch = 1;
    o->precision = PSBA_PREC_FP64;
    o->refine = 0;
}

int psba_create(const psba_problem_desc *desc, psba_handle **out)
{
    if (!out) return set_error("null output handle"), PSBA_ERR_ARG;
    *out = nullptr;
    TRY(validate(desc));
    psba_handle *h = new (std::nothrow) psba_handle();
    if (!h) return set_error("host allocation failed"), PSBA_ERR_NOMEM;
    keep_pool_memory();
    {
        const int r = prepare_device_kernels();
        if (r != PSBA_OK) {
            destroy_impl(h);
            return r;
        }
    }
    cudaError_t e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&h->ev1);
    for (int k = 0; k < ST_N && e == cudaSuccess; ++k) {
        e = cudaEventCreate(&h->timers[k].a);
        if (e == cudaSuccess) e = cudaEventCreate(&h->timers[k].b);
    }
    if (e != cudaSuccess) {
        set_error(std::string("CUDA error: ") + cudaGetErrorString(e));
        destroy_impl(h);
        return PSBA_ERR_CUDA;
    }
    const int r = create_impl(desc, h);
    if (r != PSBA_OK) {
        destroy_impl(h);
        return r;
    }
    *out = h;
    return PSBA_OK;
}

int psba_destroy(psba_handle *h)
{
    destroy_impl(h);
    return PSBA_OK;
}

int psba_get_params(psba_handle *h, double *cams, double *pts)
{
    if (!h || !cams || (h->d.np && !pts)) return set_error("null argument"), PSBA_ERR_ARG;
    PSBA_CUDA_TRY(cudaMemcpyAsync(cams, h->d.cams, sizeof(double) * h->d.N, cudaMemcpyDeviceToHost,
                                  h->stream));
    if (h->d.np)
        PSBA_CUDA_TRY(cudaMemcpyAsync(pts, h->d.pts, sizeof(double) * 3 * (size_t)h->d.np,
                                      cudaMemcpyDeviceToHost, h->stream));
    h->d2h_bytes += sizeof(double) * ((size_t)h->d.N + 3 * (size_t)h->d.np);
    return sync(h);
}

int psba_set_params(psba_handle *h, const double *cams, const double *pts)
{
    if (!h || !cams || (h->d.np && !pts)) return set_error("null argument"), PSBA_ERR_ARG;
    PSBA_CUDA_TRY(cudaMemcpyAsync(h->d.cams, cams, sizeof(double) * h->d.N, cudaMemcpyHostToDevice,
                                  h->stream));
    if (h->d.np)
        PSBA_CUDA_TRY(cudaMemcpyAsync(h->d.pts, pts, sizeof(double) * 3 * (size_t)h->d.np,
                                      cudaMemcpyHostToDevice, h->stream));
    h->linearized = 0;
    return sync(h);
}

int psba_reset_params(psba_handle *h)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    PSBA_CUDA_TRY(cudaMemcpyAsync(h->d.cams, h->d.cams0, sizeof(double) * h->d.N, cudaMemcpyDeviceToDevice,
                                  h->stream));
    if (h->d.np)
        PSBA_CUDA_TRY(cudaMemcpyAsync(h->d.pts, h->d.pts0, sizeof(double) * 3 * (size_t)h->d.np,
                                      cudaMemcpyDeviceToDevice, h->stream));
    h->linearized = 0;
    return sync(h);
}

int psba_levmar(psba_handle *h, const psba_opts *opts, int *itno, psba_result *res)
{
    if (!h || !itno) return set_error("null argument"), PSBA_ERR_ARG;
    TRY(check_opts(opts));
    h->d.prec = opts->precision;
    h->refine = opts->refine;
    reset_result(res);
    TRY(timed_begin(h));
    int flag = 0;
    TRY(levmar_impl(h, opts, itno, res, &flag));
    TRY(timed_end(h, res));
    return PSBA_OK;
}

int psba_levmar_resume(psba_handle *h, const psba_opts *opts, double mu, int nu, double p_L2, int *itno,
                       psba_result *res)
{
    if (!h || !itno) return set_error("null argument"), PSBA_ERR_ARG;
    TRY(check_opts(opts));
    if (!(mu > 0.0) || !std::isfinite(mu) || nu < 2 || !(p_L2 >= 0.0) || !std::isfinite(p_L2))
        return set_error("psba_levmar_resume: mu > 0, nu >= 2 and a finite p_L2 >= 0 are needed"), PSBA_ERR_ARG;
    h->d.prec = opts->precision;
    h->refine = opts->refine;
    reset_result(res);
    TRY(timed_begin(h));
    int flag = 0;
    const LmState st{mu, p_L2, nu};
    TRY(levmar_impl(h, opts, itno, res, &flag, &st));
    TRY(timed_end(h, res));
    return PSBA_OK;
}

int psba_trust_region(psba_handle *h, const psba_opts *opts, int *itno, psba_result *res)
{
    if (!h || !itno) return set_error("null argument"), PSBA_ERR_ARG;
    TRY(check_opts(opts));
    h->d.prec = opts->precision;
    h->refine = opts->refine;
    reset_result(res);
    TRY(timed_begin(h));
    int flag = 0;
    TRY(trust_region_impl(h, opts, itno, res, &flag));
    TRY(timed_end(h, res));
    return PSBA_OK;
}

int psba_solve_hybrid(psba_handle *h, const psba_opts *opts, psba_result *res)
{
    if (!h) return set_error("null argument"), PSBA_ERR_ARG;
    TRY(check_opts(opts));
    h->d.prec = opts->precision;
    h->refine = opts->refine;
    reset_result(res);
    TRY(timed_begin(h));
    int itno = 0, flag = 0;
    double init = NAN;
    while (true) {
        TRY(levmar_impl(h, opts, &itno, res, &flag));
        if (res && std::isnan(init)) init = res->initial_cost;
        if (flag != PSBA_ITER_TURN_TO_TR) break;
        TRY(trust_region_impl(h, opts, &itno, res, &flag));
        if (flag != PSBA_ITER_TURN_TO_LM) break;
    }
    if (res) res->initial_cost = init;
    TRY(timed_end(h, res));
    return PSBA_OK;
}

int psba_eval_residual(psba_handle *h, double *ex, double *cost)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    enqueue_cost_current(h, h->d.ex);
    TRY(check_launch());
    double sc[64];
    TRY(read_scalars(h, sc));
    if (cost) *cost = sc[SC_COST];
    if (ex && h->d.no)
        PSBA_CUDA_TRY(cudaMemcpyAsync(ex, h->d.ex, sizeof(double) * 2 * (size_t)h->d.no,
                                      cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int psba_eval_jacobian(psba_handle *h, double *JA, double *JB)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    enqueue_linearize(h, 1.0);
    h->linearized = 1;
    TRY(check_launch());
    const size_t no = (size_t)h->d.no;
    TRY(copy_out(h, JA, h->d.A, 2 * (size_t)h->d.cnp * no));
    TRY(copy_out(h, JB, h->d.B, 6 * no));
    return sync(h);
}

int psba_eval_normal(psba_handle *h, double coeff, double *U, double *V, double *W, double *g)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    DeviceProblem &d = h->d;
    enqueue_linearize(h, coeff);
    h->linearized = 1;
    TRY(check_launch());
    const size_t no = (size_t)d.no, np = (size_t)d.np;
    if (U)
        PSBA_CUDA_TRY(cudaMemcpyAsync(U, d.U, sizeof(double) * d.cnp * d.cnp * (size_t)d.nc, cudaMemcpyDeviceToHost,
                                      h->stream));
    if (V && np) {
        const int prec = d.prec;
        d.prec = PSBA_PREC_FP64;  // V is FP64 in both forms
        launch_expand_V(d, d.V, d.tmp9, h->stream);
        d.prec = prec;
        PSBA_CUDA_TRY(cudaMemcpyAsync(V, d.tmp9, sizeof(double) * 9 * np, cudaMemcpyDeviceToHost, h->stream));
    }
    TRY(copy_out(h, W, d.W, 3 * (size_t)d.cnp * no));
    if (g) PSBA_CUDA_TRY(cudaMemcpyAsync(g, d.g, sizeof(double) * (d.N + 3 * np), cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int psba_eval_reduced(psba_handle *h, double mu, double *Vinv, double *Y, double *S, double *ea)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    if (!h->linearized) return set_error("psba_eval_reduced needs a linearization first"), PSBA_ERR_STATE;
    DeviceProblem &d = h->d;
    enqueue_reduced(h, mu);
    h->last_mu = mu;
    TRY(check_launch());
    const size_t no = (size_t)d.no, np = (size_t)d.np;
    TRY(copy_out(h, Y, d.Y, 3 * (size_t)d.cnp * no));
    if (Vinv && np) {
        const int prec = d.prec;
        d.prec = PSBA_PREC_FP64;  // V^-1 is FP64 in both forms
        launch_expand_V(d, d.Vinv, d.tmp9, h->stream);
        d.prec = prec;
        PSBA_CUDA_TRY(cudaMemcpyAsync(Vinv, d.tmp9, sizeof(double) * 9 * np, cudaMemcpyDeviceToHost, h->stream));
    }
    if (S)
        PSBA_CUDA_TRY(cudaMemcpy2DAsync(S, sizeof(double) * d.N, d.S, sizeof(double) * d.Np,
                                        sizeof(double) * d.N, d.N, cudaMemcpyDeviceToHost, h->stream));
    if (ea) PSBA_CUDA_TRY(cudaMemcpyAsync(ea, d.rhs, sizeof(double) * d.N, cudaMemcpyDeviceToHost, h->stream));
    TRY(sync(h));
    if (S)
        for (int r = 0; r < d.N; ++r)
            for (int c = r + 1; c < d.N; ++c) S[(size_t)r * d.N + c] = 0.0;
    return PSBA_OK;
}

int psba_eval_step(psba_handle *h, double *dp, int *chol_status)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    if (!h->linearized) return set_error("psba_eval_step needs a reduced system first"), PSBA_ERR_STATE;
    DeviceProblem &d = h->d;
    enqueue_step(h, h->last_mu);
    TRY(check_launch());
    TrialScalars ts;
    TRY(read_trial(h, &ts));
    if (ts.chol_status == 2)
        return set_error("dense solver wait budget exhausted (device dataflow stalled)"), PSBA_ERR_STATE;
    if (chol_status) *chol_status = ts.chol_status;
    if (dp && ts.chol_status == 0)
        PSBA_CUDA_TRY(cudaMemcpyAsync(dp, d.dp, sizeof(double) * (d.N + 3 * (size_t)d.np),
                                      cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int psba_eval_jmultiply(psba_handle *h, const double *x, double *out)
{
    if (!h || !x || !out) return set_error("null argument"), PSBA_ERR_ARG;
    if (!h->linearized) return set_error("psba_eval_jmultiply needs a Jacobian first"), PSBA_ERR_STATE;
    DeviceProblem &d = h->d;
    PSBA_CUDA_TRY(cudaMemcpyAsync(d.vecP, x, sizeof(double) * (d.N + 3 * (size_t)d.np),
                                  cudaMemcpyHostToDevice, h->stream));
    launch_jmultiply(d, d.vecP, d.jx1, h->stream);
    TRY(check_launch());
    if (d.no)
        PSBA_CUDA_TRY(cudaMemcpyAsync(out, d.jx1, sizeof(double) * 2 * (size_t)d.no, cudaMemcpyDeviceToHost,
                                      h->stream));
    return sync(h);
}

int psba_eval_cholmod(int n, double *S, double *E)
{
    if (n <= 0 || n % 3 != 0 || !S || !E) return set_error("psba_eval_cholmod needs n % 3 == 0"), PSBA_ERR_ARG;
    double *dS = nullptr, *dE = nullptr, *dW = nullptr;
    const size_t nn = (size_t)n * n;
    cudaError_t e = cudaMalloc(&dS, nn * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dE, (size_t)n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dW, cholmod_work(n) * sizeof(double));
    if (e == cudaSuccess) e = cudaMemcpy(dS, S, nn * sizeof(double), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        launch_cholmod(dS, n, n, dE, dW, 0);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(S, dS, nn * sizeof(double), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess) e = cudaMemcpy(E, dE, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost);
    cudaFree(dS);
    cudaFree(dE);
    cudaFree(dW);
    if (e != cudaSuccess) return set_error(std::string("CUDA error: ") + cudaGetErrorString(e)), PSBA_ERR_CUDA;
    return PSBA_OK;
}

int psba_set_stage_timing(psba_handle *h, int enable)
{
    return psba_set_stage_mask(h, enable != 0 ? (1u << ST_N) - 1u : 0u);
}

int psba_set_stage_mask(psba_handle *h, unsigned mask)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    TRY(sync(h));
    h->timing = mask & ((1u << ST_N) - 1u);
    for (int k = 0; k < ST_N; ++k) {
        h->timers[k].pending = false;
        h->timers[k].total_ms = 0.0;
        h->timers[k].count = 0;
    }
    return PSBA_OK;
}

int psba_get_stage_timing(psba_handle *h, double *total_ms, long long *counts, int n)
{
    if (!h || !total_ms || !counts) return set_error("null argument"), PSBA_ERR_ARG;
    TRY(sync(h));
    for (int k = 0; k < n && k < ST_N; ++k) {
        total_ms[k] = h->timers[k].total_ms;
        counts[k] = h->timers[k].count;
    }
    return ST_N;
}

int psba_transfer_bytes(psba_handle *h, size_t *h2d, size_t *d2h)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    if (h2d) *h2d = h->h2d_bytes;
    if (d2h) *d2h = h->d2h_bytes;
    return PSBA_OK;
}

int psba_set_wait_limit(psba_handle *h, long long polls)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    if (polls < 0) return set_error("psba_set_wait_limit: polls must be >= 0"), PSBA_ERR_ARG;
    TRY(sync(h));
    h->d.wait_limit = polls == 0 ? DEFAULT_WAIT_LIMIT : polls;
    return PSBA_OK;
}

int psba_set_precision(psba_handle *h, int precision)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    if (precision != PSBA_PREC_FP64 && precision != PSBA_PREC_MIXED)
        return set_error("unknown precision"), PSBA_ERR_ARG;
    TRY(sync(h));
    h->d.prec = precision;
    h->linearized = 0;
    return PSBA_OK;
}

int psba_set_refine(psba_handle *h, int refine)
{
    if (!h) return set_error("null handle"), PSBA_ERR_ARG;
    if (refine != 0 && refine != 1) return set_error("refine must be 0 or 1"), PSBA_ERR_ARG;
    TRY(sync(h));
    h->refine = refine;
    return PSBA_OK;
}

const char *psba_last_error(void) { return psba::g_last_error.c_str(); }

void *psba_stream(psba_handle *h) { return h ? (void *)h->stream : nullptr; }

size_t psba_device_bytes(psba_handle *h) { return h ? h->d.bytes : 0; }

const char *psba_version(void) { return "psba_gb300 0.1 (sm_103a, FP64)"; }

}  // extern "C"

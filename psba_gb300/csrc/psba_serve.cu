// Serving engine: continuous (iteration-level) batching of independent
// bundle-adjustment requests on one GPU.
//
// A request is laid out on the submitting thread (index lists, Schur pair
// lists) and queued.  A worker thread admits queued requests in arrival order
// while a resident slot is free and the request's footprint fits the HBM
// pool (one cudaMalloc of the budget at creation, carved by a first-fit
// allocator, so admission is exactly "fits the budget").  Admitted problems
// keep parameters, linearisation and LM state (BatchResult) on the device and
// advance together in time slices: each slice is one persistent launch of the
// batched LM kernel in which every resident problem runs a number of outer LM
// iterations scaled so that all of them take about as long as the heaviest
// one's slice.  Between slices the worker retires finished problems (copies
// their parameters out, frees their memory and slot) and admits new ones,
// which join the next launch.  A problem's arithmetic depends only on its own
// data and on outer-iteration boundaries, which are where slices cut, so its
// result is the same bits alone and in any mix.
//
// Large requests (more than large_cams cameras) take the large lane instead:
// large_lanes host threads each solve one request at a time with the
// single-problem engine (psba_create / psba_levmar on its own stream: kernels
// over the whole GPU and the cooperative dataflow Cholesky), concurrently
// with the batch lane's launches, within large_share of the HBM budget; the
// batch lane's pool is the rest.  One CTA per problem would leave a
// 138-camera request with an N = 828 FP64 Cholesky on a single SM (~25 ms per
// trial); the whole GPU factors it in ~2 ms.  A dataflow wait that runs out
// of budget while the batch lane holds SMs fails that request with an error
// status (it cannot hang): waits are bounded, and slices end on their own.
//
// The per-request solve is levmar() (PSBA/levmar.cpp:45-256); the reference
// has no serving layer (one problem per process, PSBA/main.cpp:193-208).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "psba_batch_internal.h"

using namespace psba;
using namespace psba::batch;

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b)
{
    return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
    long long ticket = 0;
    ProblemLayout L;
    size_t bytes = 0;
    int slot = -1;
    size_t off = 0;
    int state = 0;  // 0 queued, 1 resident, 2 finished
    Clock::time_point t_submit, t_admit, t_done;
    BatchResult st{};
    std::vector<double> cams, pts;
    // large lane: a copy of the problem for psba_create, and the outcome
    bool large = false;
    int nc = 0, np = 0, no = 0, cnp = 6;
    std::vector<double> hK, hq0, hcams, hpts, hmeas, hcov;
    std::vector<int> hopt, hocam;
    int err = PSBA_OK;
    std::string err_msg;
};

// First-fit allocator over [0, size) in 256-byte units, coalescing on free.
class PoolAllocator {
  public:
    void reset(size_t size)
    {
        free_.clear();
        if (size) free_[0] = size;
        used_ = 0;
    }
    bool alloc(size_t bytes, size_t &off)
    {
        bytes = (bytes + 255) & ~(size_t)255;
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                off = it->first;
                const size_t rest = it->second - bytes;
                free_.erase(it);
                if (rest) free_[off + bytes] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t off, size_t bytes)
    {
        bytes = (bytes + 255) & ~(size_t)255;
        used_ -= bytes;
        auto it = free_.emplace(off, bytes).first;
        auto nx = std::next(it);
        if (nx != free_.end() && it->first + it->second == nx->first) {
            it->second += nx->second;
            free_.erase(nx);
        }
        if (it != free_.begin()) {
            auto pv = std::prev(it);
            if (pv->first + pv->second == it->first) {
                pv->second += it->second;
                free_.erase(it);
            }
        }
    }
    size_t used() const { return used_; }

  private:
    std::map<size_t, size_t> free_;
    size_t used_ = 0;
};

}  // namespace

struct psba_server {
    psba_server_opts so{};
    psba_opts lm{};
    BatchOpts bo{};
    int precision = PSBA_PREC_FP64;
    size_t rsize = sizeof(double);
    // device
    char *pool = nullptr;
    size_t pool_size = 0;
    BatchProblem *d_probs = nullptr;
    int *d_order = nullptr, *d_queue = nullptr;
    BatchResult *d_state = nullptr;
    BatchOpts *d_opts = nullptr;
    // pinned host mirrors
    BatchProblem *h_probs = nullptr;
    BatchResult *h_state = nullptr;
    int *h_order = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int device = 0, grid_cap = 1;
    int large_chol_cap = 0;  // dense-factor CTAs per large-lane solve: the SMs shared among the lanes
    // scheduling state (guarded by mu)
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    PoolAllocator alloc;
    std::deque<Request *> queue;
    std::vector<Request *> slots;
    std::unordered_map<long long, std::unique_ptr<Request>> reqs;
    long long next_ticket = 1;
    int n_active = 0;
    bool stop = false;
    int failed = 0;
    std::string fail_msg;
    psba_server_stats stats{};
    std::thread worker;
    // large lane
    std::condition_variable cv_large;
    std::deque<Request *> large_queue;
    size_t large_budget = 0, large_in_use = 0;
    int n_large = 0;  // large requests being solved
    std::vector<std::thread> large_workers;
};

namespace {

void server_fail(psba_server *s, cudaError_t e, const char *what)
{
    std::lock_guard<std::mutex> lk(s->mu);
    if (!s->failed) {
        s->failed = 1;
        s->fail_msg = std::string("psba server: ") + what + ": " + cudaGetErrorString(e);
    }
    s->cv_done.notify_all();
}

// Upload a newly admitted request into its pool region and slot.
cudaError_t upload(psba_server *s, Request *r)
{
    const ProblemLayout &L = r->L;
    const size_t d_bytes = (sizeof(double) * L.dA.size() + 255) & ~(size_t)255;
    const size_t i_bytes = (sizeof(int) * L.iA.size() + 255) & ~(size_t)255;
    BatchProblem bp = L.bp;
    rebase_problem(bp, (long long)(r->off / sizeof(double)), (long long)((r->off + d_bytes) / sizeof(int)),
                   (long long)((r->off + d_bytes + i_bytes) / s->rsize));
    bp.flags = (bp.flags & ~0xff) | (s->so.lanes_per_pair & 0xff);
    s->h_probs[r->slot] = bp;
    cudaError_t e = cudaSuccess;
    if (!L.dA.empty())
        e = cudaMemcpyAsync(s->pool + r->off, L.dA.data(), sizeof(double) * L.dA.size(), cudaMemcpyHostToDevice,
                            s->stream);
    if (e == cudaSuccess && !L.iA.empty())
        e = cudaMemcpyAsync(s->pool + r->off + d_bytes, L.iA.data(), sizeof(int) * L.iA.size(),
                            cudaMemcpyHostToDevice, s->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_state + r->slot, 0, sizeof(BatchResult), s->stream);
    return e;
}

void worker_main(psba_server *s)
{
    cudaSetDevice(s->device);
    std::vector<Request *> admitted, active, done;
    while (true) {
        admitted.clear();
        active.clear();
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || !s->queue.empty() || s->n_active > 0; });
            if (s->stop || s->failed) break;
            while (!s->queue.empty() && s->n_active < s->so.max_active) {
                Request *r = s->queue.front();
                size_t off = 0;
                if (!s->alloc.alloc(r->bytes, off)) break;  // arrival order: wait for memory
                int slot = 0;
                while (s->slots[slot]) ++slot;
                r->slot = slot;
                r->off = off;
                r->state = 1;
                r->t_admit = Clock::now();
                s->slots[slot] = r;
                s->n_active++;
                s->queue.pop_front();
                admitted.push_back(r);
                s->stats.admitted++;
            }
            s->stats.bytes_in_use = (double)s->alloc.used();
            s->stats.peak_bytes = std::max(s->stats.peak_bytes, s->stats.bytes_in_use);
            for (Request *r : s->slots)
                if (r) active.push_back(r);
        }
        if (active.empty()) continue;
        cudaError_t e = cudaSuccess;
        for (Request *r : admitted)
            if (e == cudaSuccess) e = upload(s, r);
        if (e != cudaSuccess) {
            server_fail(s, e, "upload");
            break;
        }
        // time-balanced slice: the heaviest resident problem runs slice_iters
        // outer iterations, lighter ones proportionally more
        double wmax = 0.0;
        for (Request *r : active) wmax = std::max(wmax, r->L.work);
        int max_slot = 0;
        for (Request *r : active) {
            const double k = std::floor(s->so.slice_iters * wmax / std::max(r->L.work, 1.0));
            s->h_probs[r->slot].slice = (int)std::min<double>(std::max<double>(k, s->so.slice_iters), s->bo.max_iter);
            max_slot = std::max(max_slot, r->slot + 1);
        }
        std::sort(active.begin(), active.end(), [](const Request *a, const Request *b) {
            return a->L.work > b->L.work;
        });
        for (size_t q = 0; q < active.size(); ++q) s->h_order[q] = active[q]->slot;
        const int n = (int)active.size();
        e = cudaMemcpyAsync(s->d_probs, s->h_probs, sizeof(BatchProblem) * max_slot, cudaMemcpyHostToDevice,
                            s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->d_order, s->h_order, sizeof(int) * n, cudaMemcpyHostToDevice, s->stream);
        if (e == cudaSuccess) e = cudaMemsetAsync(s->d_queue, 0, sizeof(int), s->stream);
        if (e == cudaSuccess) e = cudaEventRecord(s->ev0, s->stream);
        if (e == cudaSuccess)
            e = launch_batch_lm(s->precision, std::min(n, s->grid_cap), s->so.threads, s->stream, s->d_probs,
                                s->d_order, n, s->d_queue, (double *)s->pool, (int *)s->pool, (void *)s->pool,
                                s->d_opts, s->d_state);
        note_launch(1);
        if (e == cudaSuccess) e = cudaEventRecord(s->ev1, s->stream);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(s->h_state, s->d_state, sizeof(BatchResult) * max_slot, cudaMemcpyDeviceToHost,
                                s->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) {
            server_fail(s, e, "slice");
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, s->ev0, s->ev1);
        // retire finished problems
        done.clear();
        for (Request *r : active) {
            const BatchResult &st = s->h_state[r->slot];
            if (st.status != PSBA_ITER_CONTINUE || st.iterations >= s->bo.max_iter) {
                r->st = st;
                const BatchProblem &bp = s->h_probs[r->slot];
                r->cams.resize(6 * (size_t)bp.nc);
                r->pts.resize(3 * (size_t)bp.np);
                e = cudaMemcpyAsync(r->cams.data(), (double *)s->pool + bp.d_cams, sizeof(double) * r->cams.size(),
                                    cudaMemcpyDeviceToHost, s->stream);
                if (e == cudaSuccess && bp.np)
                    e = cudaMemcpyAsync(r->pts.data(), (double *)s->pool + bp.d_pts, sizeof(double) * r->pts.size(),
                                        cudaMemcpyDeviceToHost, s->stream);
                if (e != cudaSuccess) break;
                done.push_back(r);
            }
        }
        if (e == cudaSuccess && !done.empty()) e = cudaStreamSynchronize(s->stream);
        if (e != cudaSuccess) {
            server_fail(s, e, "retire");
            break;
        }
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->stats.launches++;
            s->stats.busy_ms += ms;
            const auto now = Clock::now();
            for (Request *r : done) {
                s->alloc.release(r->off, r->bytes);
                s->slots[r->slot] = nullptr;
                s->n_active--;
                r->slot = -1;
                r->state = 2;
                r->t_done = now;
                s->stats.finished++;
                r->L.dA.clear();
                r->L.dA.shrink_to_fit();
                r->L.iA.clear();
                r->L.iA.shrink_to_fit();
            }
            s->stats.bytes_in_use = (double)s->alloc.used();
        }
        if (!done.empty()) s->cv_done.notify_all();
    }
}

// Device bytes of a request on the single-problem engine (an upper estimate
// of what psba_create allocates): per observation e, A, B, W, Y, J x
// buffers and indices; per point V, V^-1, g, dp and trust-region vectors;
// the camera-pair entries and their Schur partials; S, its copy and the
// dense-solve work arrays; 16 MB of slack for the small tables.
size_t large_bytes(const psba_problem_desc &p, int cnp)
{
    const size_t no = (size_t)p.n_obs, np = (size_t)p.n_pts, nc = (size_t)p.n_cams, c = (size_t)cnp;
    size_t entries = 0;
    for (size_t a = 0, b = 0; a < no; a = b) {
        while (b < no && p.obs_pt[b] == p.obs_pt[a]) ++b;
        entries += (b - a) * (b - a - 1) / 2;
    }
    const size_t N = c * nc, Np = (N + TILE - 1) / TILE * TILE;
    // off-diagonal partial slots: 6-parameter cameras, one per chunk plus one
    // per pair boundary inside a chunk; otherwise one per unit
    const size_t off_units = c == 6 ? std::min(entries / OFF_MIN_LEN + 1, (size_t)schur_off_wave_threads())
                                    : entries / SCHUR_CHUNK;
    const size_t per_obs = 2 + 2 * c + 6 + 2 * 3 * c + 3 * 2 + 3 + 4;
    const size_t per_pt = 3 * 3 + 6 * 2 + 9 + 3 * 6;
    const size_t doubles = no * per_obs + np * per_pt + N * 8 + nc * (c * c + 2 * CAMTAB) + 3 * Np * Np +
                           Np * TILE + (off_units + nc * 8) * c * c +
                           (no / (c == 6 ? DIAG_SUPER : DIAG_CHUNK) + nc) * (c * (c + 1) / 2 + c);  // diagonal-unit partials
    // index-build scratch: counts and offsets per (pair-list segment, camera)
    const size_t segs = no / (size_t)pair_segment_len(p.n_cams, p.n_obs) + nc;
    return doubles * sizeof(double) + entries * 2 * sizeof(int) + segs * nc * 2 * sizeof(int) + ((size_t)16 << 20);
}

void large_main(psba_server *s)
{
    cudaSetDevice(s->device);
    while (true) {
        Request *r = nullptr;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_large.wait(lk, [&] {
                return s->stop ||
                       (!s->large_queue.empty() && s->large_in_use + s->large_queue.front()->bytes <= s->large_budget);
            });
            if (s->stop) break;
            r = s->large_queue.front();
            s->large_queue.pop_front();
            s->large_in_use += r->bytes;
            r->state = 1;
            r->t_admit = Clock::now();
            s->stats.admitted++;
            s->n_large++;
        }
        psba_problem_desc desc{};
        desc.n_cams = r->nc;
        desc.n_pts = r->np;
        desc.n_obs = r->no;
        desc.K = r->hK.data();
        desc.q0 = r->hq0.data();
        desc.cams = r->hcams.data();
        desc.pts = r->hpts.data();
        desc.meas = r->hmeas.data();
        desc.obs_pt = r->hopt.data();
        desc.obs_cam = r->hocam.data();
        desc.cnp = r->cnp;
        desc.cov = r->hcov.empty() ? nullptr : r->hcov.data();
        psba_handle *h = nullptr;
        psba_result res{};
        int itno = 0;
        int rc = psba_create(&desc, &h);
        // the lanes' dense factors run side by side: each takes its share of the SMs
        if (rc == PSBA_OK) set_chol_grid_cap(h, s->large_chol_cap);
        if (rc == PSBA_OK && s->so.large_wait_limit > 0) rc = psba_set_wait_limit(h, s->so.large_wait_limit);
        // cameras with intrinsics (11/16 parameters) in FP64 when the server
        // asks for it: their mixed-form Jacobian columns lose the
        // ill-conditioned intrinsics directions (slow or stalled convergence)
        psba_opts lm = s->lm;
        if (r->cnp != 6 && s->so.fp64_intrinsics) lm.precision = PSBA_PREC_FP64;
        if (rc == PSBA_OK) rc = psba_levmar(h, &lm, &itno, &res);
        r->cams.resize((size_t)r->cnp * r->nc);
        r->pts.resize(3 * (size_t)r->np);
        if (rc == PSBA_OK) rc = psba_get_params(h, r->cams.data(), r->pts.data());
        const double dev_bytes = h ? (double)psba_device_bytes(h) : 0.0;
        const std::string msg = rc == PSBA_OK ? std::string() : std::string(psba_last_error());
        if (h) psba_destroy(h);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->large_in_use -= r->bytes;
            s->n_large--;
            r->st.status = res.status;
            r->st.iterations = res.iterations;
            r->st.trials = res.n_trials;
            r->st.linearizations = res.n_linearizations;
            r->st.initial_cost = res.initial_cost;
            r->st.final_cost = res.final_cost;
            r->err = rc;
            r->err_msg = msg;
            if (dev_bytes > 0) r->bytes = (size_t)dev_bytes;
            r->state = 2;
            r->t_done = Clock::now();
            s->stats.finished++;
            for (std::vector<double> *v : {&r->hK, &r->hq0, &r->hcams, &r->hpts, &r->hmeas, &r->hcov})
                std::vector<double>().swap(*v);
            std::vector<int>().swap(r->hopt);
            std::vector<int>().swap(r->hocam);
        }
        s->cv_done.notify_all();
        s->cv_large.notify_all();
    }
}

void server_free(psba_server *s)
{
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    s->cv_large.notify_all();
    if (s->worker.joinable()) s->worker.join();
    for (std::thread &t : s->large_workers)
        if (t.joinable()) t.join();
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->pool);
    cudaFree(s->d_probs);
    cudaFree(s->d_order);
    cudaFree(s->d_queue);
    cudaFree(s->d_state);
    cudaFree(s->d_opts);
    cudaFreeHost(s->h_probs);
    cudaFreeHost(s->h_state);
    cudaFreeHost(s->h_order);
    if (s->ev0) cudaEventDestroy(s->ev0);
    if (s->ev1) cudaEventDestroy(s->ev1);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

}  // namespace

extern "C" {

void psba_server_default_opts(psba_server_opts *o)
{
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->hbm_budget_bytes = 120e9;
    o->max_active = 1024;
    o->slice_iters = 1;
    o->threads = 256;
    o->lanes_per_pair = 32;
    o->large_cams = 40;
    o->large_lanes = 8;
    o->large_share = 0.25;
    o->large_obs = 20000;
    o->fp64_intrinsics = 1;
}

int psba_server_create(const psba_server_opts *so, const psba_opts *lm, psba_server **out)
{
    if (!so || !lm || !out) return set_error("psba_server_create: null argument"), PSBA_ERR_ARG;
    *out = nullptr;
    if (so->hbm_budget_bytes < 1e6 || so->max_active < 1 || so->max_active > 65536 || so->slice_iters < 1 ||
        (so->threads != 128 && so->threads != 256 && so->threads != 512) ||
        (so->lanes_per_pair != 8 && so->lanes_per_pair != 16 && so->lanes_per_pair != 32) || so->large_cams < 0 ||
        so->large_lanes < 0 || so->large_lanes > 16 || !(so->large_share >= 0.0 && so->large_share < 1.0) ||
        so->large_obs < 0 || so->large_wait_limit < 0 || so->large_chol_ctas < 0 ||
        (lm->precision != PSBA_PREC_FP64 && lm->precision != PSBA_PREC_MIXED) || lm->max_iter < 0 ||
        lm->refine != 0)
        return set_error("psba_server_create: bad options"), PSBA_ERR_ARG;
    psba_server *s = new psba_server();
    s->so = *so;
    s->lm = *lm;
    s->lm.allow_switch = 0;
    s->precision = lm->precision;
    s->rsize = lm->precision == PSBA_PREC_MIXED ? sizeof(float) : sizeof(double);
    s->bo.tau = lm->tau;
    s->bo.stop_thresh = lm->stop_thresh;
    s->bo.eps = lm->eps;
    s->bo.max_iter = lm->max_iter;
    s->bo.allow_switch = 0;  // the batched driver is LM only
    s->bo.precision = lm->precision;
    const bool with_large = so->large_cams > 0 && so->large_lanes > 0;
    s->large_budget = with_large ? (size_t)(so->hbm_budget_bytes * so->large_share) : 0;
    s->pool_size = (size_t)(so->hbm_budget_bytes - (double)s->large_budget) & ~(size_t)255;
    const int M = so->max_active;
    cudaError_t e = cudaGetDevice(&s->device);
    int sms = 1;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, s->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&s->ev1);
    if (e == cudaSuccess) e = cudaMalloc(&s->pool, s->pool_size);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_probs, sizeof(BatchProblem) * M);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_order, sizeof(int) * M);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_queue, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&s->d_state, sizeof(BatchResult) * M);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_opts, sizeof(BatchOpts));
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_probs, sizeof(BatchProblem) * M);
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_state, sizeof(BatchResult) * M);
    if (e == cudaSuccess) e = cudaMallocHost(&s->h_order, sizeof(int) * M);
    if (e == cudaSuccess) e = cudaMemcpy(s->d_opts, &s->bo, sizeof(BatchOpts), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        set_error(std::string("psba_server_create: ") + cudaGetErrorString(e));
        server_free(s);
        return e == cudaErrorMemoryAllocation ? PSBA_ERR_NOMEM : PSBA_ERR_CUDA;
    }
    std::memset(s->h_probs, 0, sizeof(BatchProblem) * M);
    s->grid_cap = batch_blocks_per_sm(s->precision, so->threads) * sms;
    if (with_large)
        s->large_chol_cap = so->large_chol_ctas > 0 ? std::min(so->large_chol_ctas, sms)
                                                    : std::max(2, sms / so->large_lanes);
    s->alloc.reset(s->pool_size);
    s->slots.assign(M, nullptr);
    s->worker = std::thread(worker_main, s);
    if (with_large)
        for (int k = 0; k < so->large_lanes; ++k) s->large_workers.emplace_back(large_main, s);
    *out = s;
    return PSBA_OK;
}

int psba_batch_submit(psba_server *s, const psba_problem_desc *desc, long long *ticket)
{
    if (!s || !desc || !ticket) return set_error("psba_batch_submit: null argument"), PSBA_ERR_ARG;
    auto r = std::make_unique<Request>();
    r->t_submit = Clock::now();
    const int cnp = desc->cnp == 0 ? 6 : desc->cnp;
    // the batch lane takes 6-parameter, unweighted problems; the others, and
    // those above large_cams cameras, go to the single-problem engine
    const bool special = cnp != 6 || desc->cov != nullptr;
    if (special && s->large_budget == 0)
        return set_error("psba_batch_submit: 11/16-parameter cameras and weighted problems need the large lane "
                         "(large_cams > 0, large_lanes > 0)"),
               PSBA_ERR_ARG;
    r->large = s->large_budget > 0 && (special || desc->n_cams > s->so.large_cams ||
                                       (s->so.large_obs > 0 && desc->n_obs > s->so.large_obs));
    if (r->large) {
        // checked in full by psba_create on the large lane; enough here to copy safely
        if ((cnp != 6 && cnp != 11 && cnp != 16) || desc->n_cams <= 0 || desc->n_pts < 0 || desc->n_obs < 0 ||
            (cnp == 6 && !desc->K) || !desc->q0 || !desc->cams || (desc->n_pts && !desc->pts) ||
            (desc->n_obs && (!desc->meas || !desc->obs_pt || !desc->obs_cam)))
            return set_error("psba_batch_submit: problem is malformed"), PSBA_ERR_ARG;
        r->bytes = large_bytes(*desc, cnp);
        if (r->bytes > s->large_budget)
            return set_error("psba_batch_submit: the problem alone exceeds the large lane's HBM share"),
                   PSBA_ERR_NOMEM;
        // the single-problem engine lays the problem out itself: keep the input
        r->nc = desc->n_cams;
        r->np = desc->n_pts;
        r->no = desc->n_obs;
        r->cnp = cnp;
        if (desc->K) r->hK.assign(desc->K, desc->K + 5 * (size_t)r->nc);
        else r->hK.assign(5 * (size_t)r->nc, 0.0);
        r->hq0.assign(desc->q0, desc->q0 + 4 * (size_t)r->nc);
        r->hcams.assign(desc->cams, desc->cams + (size_t)cnp * r->nc);
        if (r->np) r->hpts.assign(desc->pts, desc->pts + 3 * (size_t)r->np);
        if (r->no) {
            r->hmeas.assign(desc->meas, desc->meas + 2 * (size_t)r->no);
            r->hopt.assign(desc->obs_pt, desc->obs_pt + r->no);
            r->hocam.assign(desc->obs_cam, desc->obs_cam + r->no);
            if (desc->cov) r->hcov.assign(desc->cov, desc->cov + 4 * (size_t)r->no);
        }
    } else {
        std::string err;
        if (!build_problem_layout(*desc, r->L, err)) return set_error("psba_batch_submit: " + err), PSBA_ERR_ARG;
        r->bytes = pool_bytes(r->L, s->precision);
        if (r->bytes > s->pool_size)
            return set_error("psba_batch_submit: the problem alone exceeds the HBM budget"), PSBA_ERR_NOMEM;
    }
    const bool large = r->large;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->failed) return set_error(s->fail_msg), PSBA_ERR_CUDA;
        r->ticket = s->next_ticket++;
        *ticket = r->ticket;
        if (large)
            s->large_queue.push_back(r.get());
        else
            s->queue.push_back(r.get());
        s->reqs.emplace(r->ticket, std::move(r));
        s->stats.submitted++;
    }
    if (large)
        s->cv_large.notify_all();
    else
        s->cv_work.notify_one();
    return PSBA_OK;
}

int psba_batch_poll(psba_server *s, long long ticket, int timeout_ms, psba_request_result *res, double *cams,
                    double *pts)
{
    if (!s || timeout_ms < 0) return set_error("psba_batch_poll: bad arguments"), PSBA_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->reqs.find(ticket);
    if (it == s->reqs.end()) return set_error("psba_batch_poll: unknown ticket"), PSBA_ERR_ARG;
    Request *r = it->second.get();
    const auto ready = [&] { return r->state == 2 || s->failed; };
    if (!ready() && timeout_ms > 0) s->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), ready);
    if (r->state != 2) {
        if (s->failed) return set_error(s->fail_msg), PSBA_ERR_CUDA;
        return PSBA_PENDING;
    }
    if (r->err != PSBA_OK) {
        set_error("psba_batch_poll: request failed: " + r->err_msg);
        if (res) {
            *res = psba_request_result{};
            res->status = r->err;
            res->queued_ms = ms_between(r->t_submit, r->t_admit);
            res->latency_ms = ms_between(r->t_submit, r->t_done);
        }
        s->reqs.erase(it);
        return PSBA_REQUEST_FAILED;
    }
    if (res) {
        res->status = r->st.status;
        res->iterations = r->st.iterations;
        res->n_trials = r->st.trials;
        res->n_linearizations = r->st.linearizations;
        res->initial_cost = r->st.initial_cost;
        res->final_cost = r->st.final_cost;
        res->queued_ms = ms_between(r->t_submit, r->t_admit);
        res->latency_ms = ms_between(r->t_submit, r->t_done);
        res->device_bytes = (double)r->bytes;
    }
    if (cams) std::memcpy(cams, r->cams.data(), sizeof(double) * r->cams.size());
    if (pts && !r->pts.empty()) std::memcpy(pts, r->pts.data(), sizeof(double) * r->pts.size());
    s->reqs.erase(it);
    return PSBA_OK;
}

int psba_server_stats_get(psba_server *s, psba_server_stats *st)
{
    if (!s || !st) return set_error("psba_server_stats_get: null argument"), PSBA_ERR_ARG;
    std::lock_guard<std::mutex> lk(s->mu);
    *st = s->stats;
    st->active = s->n_active + s->n_large;
    st->queued = (int)(s->queue.size() + s->large_queue.size());
    return s->failed ? (set_error(s->fail_msg), PSBA_ERR_CUDA) : PSBA_OK;
}

int psba_server_destroy(psba_server *s)
{
    server_free(s);
    return PSBA_OK;
}

}  // extern "C"

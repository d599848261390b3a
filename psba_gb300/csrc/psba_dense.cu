// Dense FP64 reduced-camera solve on sm_103a.
//
// S (Np x Np, lower triangle, Np a multiple of TILE) is factored S = L L^T
// by one cooperative persistent kernel that runs a tile dataflow: every
// TILE x TILE lower tile is a task; tasks are numbered column by column and
// each CTA takes tasks c, c + G, c + 2G, ... in increasing order.  A task
// waits (bounded spin on per-task flags in global memory, acquire/release)
// only for tasks with smaller numbers, so with all CTAs resident (cooperative
// launch) the smallest unfinished task can always run: no deadlock.
//   tile (I,I):  A_II -= sum_J L_IJ L_IJ^T, then a CTA-wide Cholesky of the
//                tile, its inverse, and y_I = L_II^-1 (b_I - sum_J L_IJ y_J)
//                (the forward solve of L y = ea rides along)
//   tile (I,K):  A_IK -= sum_{J<K} L_IJ L_KJ^T, then L_IK = A_IK L_KK^-T
// After the factor, k_tri_solve (one CTA of 512 threads, one column of the
// update per thread) solves L^T x = y with y in shared memory; the
// refinement solve of the mixed form (mode 1) runs both triangular solves
// there the same way.
//
// This replaces the reference's explicit inverse (SPD_inv.cl: 3x3-block
// Cholesky chain, kern_trigMat_inv, kern_trigMat_mul, then matVec_mul) with
// two triangular solves.  The failure test is the reference's: a non-positive
// or non-finite pivot (SPD_inv.cl:66-107) sets status 1; every task still
// raises its flag, so nothing waits forever.  A spin that runs out of its
// iteration budget sets status 2 and the kernel completes.
#include "psba_internal.h"

namespace psba {

constexpr int T = TILE;
constexpr int TT = TILE * TILE;
// Launch shape (compile-time tuning knobs): threads per CTA, update steps
// staged per batch, a cap on CTAs per SM (0: as many as fit), and whether
// CTAs claim tasks through an atomic counter (1) or take every grid-th task (0).
#ifndef PSBA_CHOL_THREADS
#define PSBA_CHOL_THREADS 128
#endif
#ifndef PSBA_CHOL_BJ
#define PSBA_CHOL_BJ 8
#endif
#ifndef PSBA_CHOL_PER_SM
#define PSBA_CHOL_PER_SM 0
#endif
#ifndef PSBA_CHOL_DYNAMIC
#define PSBA_CHOL_DYNAMIC 0
#endif
constexpr int CF_THREADS = PSBA_CHOL_THREADS;
constexpr long long SPIN_LIMIT = 1LL << 22;  // ~0.5 s of polling with 64 ns sleeps
constexpr int MAX_NP = 4096;                 // largest reduced system (dynamic shared memory of the solve)
constexpr int BJ = PSBA_CHOL_BJ;             // update steps staged per batch in a tile task
static_assert(BJ >= 2, "the diagonal factor reuses two staging tiles");

#ifdef PSBA_CHOL_TRACE
// Timing probe (off in the library): per task, the global timer at its
// start, after its updates, after its factor / triangular solve, at its end.
__device__ long long g_chol_trace[4 * 65536];
__device__ __forceinline__ void trace_mark(int t, int k)
{
    if (threadIdx.x == 0 && t < 65536) {
        long long v;
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(v));
        g_chol_trace[4 * t + k] = v;
    }
}
#define CHOL_MARK(t, k) trace_mark(t, k)
#else
#define CHOL_MARK(t, k)
#endif

__device__ __forceinline__ int ld_acquire(const int *p)
{
    int v;
    asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ void st_release(int *p, int v)
{
    asm volatile("st.release.gpu.global.s32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

// Thread 0 waits for flag == epoch; the block then proceeds.  Returns false
// when the budget ran out or another task already reported a timeout.
__device__ bool block_wait(const int *flag, int epoch, int *status)
{
    __shared__ int ok;
    if (threadIdx.x == 0) {
        int good = 0;
        for (long long it = 0; it < SPIN_LIMIT; ++it) {
            if (ld_acquire(flag) == epoch) {
                good = 1;
                break;
            }
            if (ld_acquire(status) == 2) break;
            __nanosleep(64);
        }
        if (!good) atomicExch(status, 2);
        ok = good;
    }
    __syncthreads();
    const bool r = ok != 0;
    __syncthreads();
    return r;
}

__device__ __forceinline__ int tile_task(int I, int K, int nb)
{
    return K * nb - (K * (K - 1)) / 2 + (I - K);  // column-major over the lower triangle
}

__device__ __forceinline__ void load_tile(double (*dst)[T + 1], const double *S, int Np, int I, int K)
{
    for (int e = threadIdx.x; e < TT; e += CF_THREADS) {
        const int r = e / T, c = e % T;
        dst[r][c] = __ldcg(S + (size_t)(I * T + r) * Np + K * T + c);
    }
}

// All threads: Cholesky of the lower triangle of a (T x T, shared memory),
// the factor into l (zero above the diagonal), its inverse into linv,
// invd[k] = 1 / L_kk and y = L^-1 b.  Column s: the pivot from a[s][s], column
// s of L, and the trailing update a[r][j] -= a[r][s] a[j][s] / a[s][s] for
// s < j <= r; the inverse follows one column behind (right-looking:
// X[k][.] = acc[k][.] / L_kk, acc[i][.] -= L[i][k] X[k][.] for i > k).  One
// barrier per column, and each thread does at most two trailing updates and
// one inverse update per column: on a GPU whose FP64 pipe takes tens of
// cycles per warp instruction, the chain a single warp would run (~270
// dependent FP64 operations) is what bounds the whole dense solve.
// Returns false on a non-positive or non-finite pivot.
__device__ bool cta_potrf(double (*a)[T + 1], double (*l)[T + 1], double (*acc)[T + 1], double (*linv)[T + 1],
                          double *invd, const double *b, double *y)
{
    __shared__ int bad;
    const int tid = threadIdx.x;
    for (int e = tid; e < TT; e += CF_THREADS) {
        const int r = e / T, c = e % T;
        l[r][c] = 0.0;
        linv[r][c] = 0.0;
        acc[r][c] = r == c ? 1.0 : 0.0;
    }
    if (tid == 0) bad = 0;
    __syncthreads();
    for (int s = 0; s <= T; ++s) {
        if (s < T) {
            const double d = a[s][s];
            const double inv = rsqrt(d), inv2 = inv * inv;
            if (tid == 0) {
                invd[s] = inv;
                if (!(d > 0.0) || !isfinite(d)) bad = 1;
            }
            // lower-triangle entries (r, j) with j >= s, numbered by column
            // from the right: column T-1-q holds entries q(q+1)/2 .. (q+1)(q+2)/2 - 1
            const int m = (T - s) * (T - s + 1) / 2;
            for (int e = tid; e < m; e += CF_THREADS) {
                int q = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
                while ((q + 1) * (q + 2) / 2 <= e) ++q;
                while (q * (q + 1) / 2 > e) --q;
                const int j = T - 1 - q, r = j + (e - q * (q + 1) / 2);
                if (j == s)
                    l[r][s] = r == s ? d * inv : a[r][s] * inv;
                else
                    a[r][j] = fma(-a[r][s], a[j][s] * inv2, a[r][j]);
            }
        }
        if (s >= 1) {
            const int k = s - 1;
            const double ik = invd[k];
            const int n = (T - k) * (k + 1);
            for (int e = tid; e < n; e += CF_THREADS) {
                const int i = k + e / (k + 1), c = e % (k + 1);
                const double xk = acc[k][c] * ik;
                if (i == k)
                    linv[k][c] = xk;
                else
                    acc[i][c] = fma(-l[i][k], xk, acc[i][c]);
            }
        }
        __syncthreads();
    }
    if (tid < T) {
        double sum = 0.0;
        for (int k = 0; k <= tid; ++k) sum = fma(linv[tid][k], b[k], sum);
        y[tid] = sum;
    }
    __syncthreads();
    return bad == 0;
}

// Single-CTA triangular solves over the factor (S lower = L, Linv = diagonal
// tile inverses) with the right-hand side in shared memory.  Each column step
// reads one row panel of L with coalesced loads (16 independent loads per
// thread), so a step costs about one L2 round trip.
// forward: b <- L^-1 b (right-looking: y_K = Linv_K b_K, then b_I -= L_IK y_K)
__device__ void cta_forward(int Np, int nb, const double *__restrict__ S, const double *__restrict__ Linv,
                            double *bs, double *tmp)
{
    const int tid = threadIdx.x;
    for (int K = 0; K < nb; ++K) {
        if (tid < T) {
            const double *Li = Linv + (size_t)K * TT + tid * T;
            double y = 0.0;
#pragma unroll
            for (int k = 0; k < T; ++k) y = fma(k <= tid ? __ldcg(Li + k) : 0.0, bs[K * T + k], y);
            tmp[tid] = y;
        }
        __syncthreads();
        if (tid < T) bs[K * T + tid] = tmp[tid];
        for (int i = (K + 1) * T + tid; i < Np; i += blockDim.x) {
            const double2 *row = reinterpret_cast<const double2 *>(S + (size_t)i * Np + K * T);
            double s = 0.0;
#pragma unroll
            for (int c = 0; c < T / 2; ++c) {
                const double2 v = __ldcg(row + c);
                s = fma(v.x, tmp[2 * c], s);
                s = fma(v.y, tmp[2 * c + 1], s);
            }
            bs[i] -= s;
        }
        __syncthreads();
    }
}

// back: x <- L^-T y (right-looking over the columns of L^T: x_K = Linv_K^T y_K,
// then y_I -= L_KI^T x_K for I < K, reading rows K*T..K*T+T-1 of L).
__device__ void cta_back(int Np, int nb, const double *__restrict__ S, const double *__restrict__ Linv,
                         double *ys, double *xs, double *__restrict__ x)
{
    const int tid = threadIdx.x;
    for (int K = nb - 1; K >= 0; --K) {
        if (tid < T) {
            const double *Li = Linv + (size_t)K * TT;
            double v = 0.0;
#pragma unroll
            for (int k = 0; k < T; ++k) v = fma(k >= tid ? __ldcg(Li + k * T + tid) : 0.0, ys[K * T + k], v);
            xs[tid] = v;
            x[K * T + tid] = v;
        }
        __syncthreads();
        for (int col = tid; col < K * T; col += blockDim.x) {
            const double *base = S + (size_t)(K * T) * Np + col;
            double v[T];
#pragma unroll
            for (int c = 0; c < T; ++c) v[c] = __ldcg(base + (size_t)c * Np);
            double s = 0.0;
#pragma unroll
            for (int c = 0; c < T; ++c) s = fma(v[c], xs[c], s);
            ys[col] -= s;
        }
        __syncthreads();
    }
}

// The factor (tile dataflow) with the forward solve of rhs carried along on
// the diagonal tasks; the back solve runs after it in k_tri_solve.
__global__ void __launch_bounds__(CF_THREADS) k_chol_dataflow(int Np, int nb,
                                                              const int2 *__restrict__ tasks,
                                                              double *__restrict__ S,
                                                              double *__restrict__ Linv,
                                                              double *__restrict__ rhs,
                                                              int *__restrict__ flags, int epoch,
                                                              int *__restrict__ status)
{
    __shared__ double a[T][T + 1], linv[T][T + 1];
    __shared__ double bi[BJ][T][T + 1], bk[BJ][T][T + 1], by[BJ][T];
    __shared__ double bvec[T], yvec[T], invd[T];
    __shared__ int ready_n;
    const int n_fact = nb * (nb + 1) / 2;
    const int n_tasks = n_fact;
    const int tid = threadIdx.x;
#if PSBA_CHOL_DYNAMIC
    // tasks claimed in increasing order: the smallest unfinished claimed task
    // has all its (smaller) dependencies claimed, so it can always run
    __shared__ int claim;
    while (true) {
        if (tid == 0) claim = atomicAdd(status + 1, 1);
        __syncthreads();
        const int t = claim;
        __syncthreads();
        if (t >= n_tasks) break;
#else
    for (int t = blockIdx.x; t < n_tasks; t += gridDim.x) {
#endif
        if (t < n_fact) {
            CHOL_MARK(t, 0);
            const int I = tasks[t].x, K = tasks[t].y;
            load_tile(a, S, Np, I, K);
            if (I == K && tid < T) bvec[tid] = __ldcg(rhs + I * T + tid);
            __syncthreads();
            // Updates J = 0 .. K-1 in order.  The flags of the next BJ steps are
            // polled at once (one L2 round trip); the ready ones have all their
            // tiles loaded together and are applied from shared memory, so an
            // update costs one round trip per batch instead of two per step.
            // Each thread updates its own elements in the same order as one
            // step at a time would: the arithmetic does not depend on batching.
            int J = 0;
            while (J < K) {
                const int nmax = min(BJ, K - J);
                if (tid == 0) ready_n = nmax;
                __syncthreads();
                if (tid < nmax) {
                    const bool ok = ld_acquire(flags + tile_task(I, J + tid, nb)) == epoch &&
                                    (I == K || ld_acquire(flags + tile_task(K, J + tid, nb)) == epoch);
                    if (!ok) atomicMin(&ready_n, tid);
                }
                __syncthreads();
                int n = ready_n;
                if (n == 0) {  // the next step is not done yet: wait for it alone
                    block_wait(flags + tile_task(I, J, nb), epoch, status);
                    if (I != K) block_wait(flags + tile_task(K, J, nb), epoch, status);
                    n = 1;
                }
                for (int e = tid; e < n * TT; e += CF_THREADS) {
                    const int q = e / TT, r = (e % TT) / T, c = e % T;
                    bi[q][r][c] = __ldcg(S + (size_t)(I * T + r) * Np + (J + q) * T + c);
                    if (I != K) bk[q][r][c] = __ldcg(S + (size_t)(K * T + r) * Np + (J + q) * T + c);
                }
                if (I == K)
                    for (int e = tid; e < n * T; e += CF_THREADS) by[e / T][e % T] = __ldcg(rhs + (J + e / T) * T + e % T);
                __syncthreads();
                for (int q = 0; q < n; ++q) {
                    double(*lip)[T + 1] = bi[q];
                    double(*lkp)[T + 1] = I == K ? bi[q] : bk[q];
                    for (int e = tid; e < TT; e += CF_THREADS) {
                        const int r = e / T, c = e % T;
                        double s = a[r][c];
#pragma unroll
                        for (int k = 0; k < T; ++k) s = fma(-lip[r][k], lkp[c][k], s);
                        a[r][c] = s;
                    }
                    if (I == K && tid < T) {
                        double s = bvec[tid];
#pragma unroll
                        for (int k = 0; k < T; ++k) s = fma(-lip[tid][k], by[q][k], s);
                        bvec[tid] = s;
                    }
                }
                __syncthreads();
                J += n;
            }
            CHOL_MARK(t, 1);
            const bool failed = ld_acquire(status) != 0;
            if (I == K) {
                if (!failed) {
                    // the staging tiles are free now: L in bi[0], the inverse's accumulator in bi[1]
                    const bool good = cta_potrf(a, bi[0], bi[1], linv, invd, bvec, yvec);
                    if (tid == 0 && !good) atomicCAS(status, 0, 1);
                    for (int e = tid; e < TT; e += CF_THREADS) {
                        const int r = e / T, c = e % T;
                        S[(size_t)(I * T + r) * Np + I * T + c] = bi[0][r][c];
                        Linv[(size_t)I * TT + e] = linv[r][c];
                    }
                    if (tid < T) rhs[I * T + tid] = yvec[tid];
                }
            } else {
                block_wait(flags + tile_task(K, K, nb), epoch, status);
                for (int e = tid; e < TT; e += CF_THREADS) linv[e / T][e % T] = __ldcg(Linv + (size_t)K * TT + e);
                __syncthreads();
                if (ld_acquire(status) == 0) {
                    for (int e = tid; e < TT; e += CF_THREADS) {
                        const int r = e / T, c = e % T;
                        double s = 0.0;
                        for (int k = 0; k <= c; ++k) s = fma(a[r][k], linv[c][k], s);
                        S[(size_t)(I * T + r) * Np + K * T + c] = s;
                    }
                }
            }
            CHOL_MARK(t, 2);
            __syncthreads();
            if (tid == 0) {
                __threadfence();
                st_release(flags + t, epoch);
            }
            CHOL_MARK(t, 3);
        }
        __syncthreads();
    }
}

int chol_grid(int n_tasks)
{
    static int per_sm = -1, sms = 0;
    if (per_sm < 0) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_chol_dataflow, CF_THREADS, 0);
        if (per_sm < 1) per_sm = 1;
        if (PSBA_CHOL_PER_SM > 0 && per_sm > PSBA_CHOL_PER_SM) per_sm = PSBA_CHOL_PER_SM;
    }
    const int cap = per_sm * sms;
    return n_tasks < cap ? n_tasks : cap;
}

// Triangular solves in one CTA of TS_THREADS threads with the right-hand side
// in shared memory: forward = 1 solves L y = rhs then L^T x = y (the
// refinement solve), forward = 0 only L^T x = rhs (after the factor, whose
// diagonal tasks already applied L^-1).  A failed factor (status != 0)
// leaves x untouched.
constexpr int TS_THREADS = 512;

__global__ void __launch_bounds__(TS_THREADS) k_tri_solve(int forward, int Np, int nb, const double *__restrict__ S,
                                                           const double *__restrict__ Linv,
                                                           const double *__restrict__ rhs, double *__restrict__ x,
                                                           const int *__restrict__ status)
{
    extern __shared__ double vec[];  // Np
    __shared__ double tmp[T];
    if (*status != 0) return;
    for (int i = threadIdx.x; i < Np; i += blockDim.x) vec[i] = rhs[i];
    __syncthreads();
    if (forward) cta_forward(Np, nb, S, Linv, vec, tmp);
    cta_back(Np, nb, S, Linv, vec, tmp, x);
}

void launch_chol_dataflow(const DeviceProblem &d, int mode, int epoch, double *x_out, cudaStream_t s)
{
    int nb = d.Np / T;
    int Np = d.Np;
    if (mode == 0) {
        const int grid = chol_grid(nb * (nb + 1) / 2);
        const int2 *tasks = d.chol_tasks;
        double *S = d.S, *Linv = d.Linv, *rhs = d.rhs;
        int *flags = d.chol_flags, *status = d.status;
        void *args[] = {&Np, &nb, (void *)&tasks, &S, &Linv, &rhs, &flags, &epoch, &status};
        cudaMemsetAsync(d.status, 0, 2 * sizeof(int), s);  // result word and task claim counter
        cudaLaunchCooperativeKernel((const void *)k_chol_dataflow, dim3(grid), dim3(CF_THREADS), args, 0, s);
        note_launch(1);
    }
    k_tri_solve<<<1, TS_THREADS, sizeof(double) * Np, s>>>(mode == 1, Np, nb, d.S, d.Linv, d.rhs, x_out, d.status);
    note_launch(1);
}

// Iterative refinement residual r = b - S x with the symmetric S given by its
// lower triangle (one warp per row, lanes over columns, fixed-order warp sum).
__global__ void k_refine_residual(int Np, const double *__restrict__ S, const double *__restrict__ x,
                                  const double *__restrict__ b, double *__restrict__ r)
{
    const int row = blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32;
    const int lane = threadIdx.x % 32;
    if (row >= Np) return;
    double s = 0.0;
    for (int c = lane; c < Np; c += 32) {
        const double v = c <= row ? S[(size_t)row * Np + c] : S[(size_t)c * Np + row];
        s = fma(v, x[c], s);
    }
    for (int off = 16; off > 0; off >>= 1) s += __shfl_down_sync(0xffffffffu, s, off);
    if (lane == 0) r[row] = b[row] - s;
}

__global__ void k_add_inplace(int n, double *x, const double *dx)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) x[i] = x[i] + dx[i];
}

void launch_refine(const DeviceProblem &d, int epoch, cudaStream_t s)
{
    // r = rhs_save - Ssave x  (into rhs), solve with the existing factor into xref, x += xref
    k_refine_residual<<<(d.Np + 7) / 8, 256, 0, s>>>(d.Np, d.Ssave, d.xsol, d.rhs_save, d.rhs);
    note_launch(1);
    launch_chol_dataflow(d, 1, epoch, d.xref, s);
    k_add_inplace<<<(d.Np + 255) / 256, 256, 0, s>>>(d.Np, d.xsol, d.xref);
    note_launch(1);
}

// ---------------------------------------------------------------------------
// Modified Cholesky (trust-region lambda fallback), restating cholmod_blk.cl
// with get_delta_beta (cl_cholmod.cpp:109-165) and kern_cholmod_E: block
// columns of 3 are factored as plain 3x3 blocks when the pivots are positive
// and every entry below is <= beta; otherwise their columns are redone one
// at a time with d = max(|c|, delta) and the theta/beta bound.  One block of
// threads; this path runs at most a few times per solve.
constexpr int CM_THREADS = 1024;

__device__ double block_max(double v, double *red)
{
    red[threadIdx.x] = v;
    __syncthreads();
    for (int st = CM_THREADS / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] = fmax(red[threadIdx.x], red[threadIdx.x + st]);
        __syncthreads();
    }
    const double r = red[0];
    __syncthreads();
    return r;
}

__device__ int block_or(int v, int *red)
{
    red[threadIdx.x] = v;
    __syncthreads();
    for (int st = CM_THREADS / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] = red[threadIdx.x] | red[threadIdx.x + st];
        __syncthreads();
    }
    const int r = red[0];
    __syncthreads();
    return r;
}

__global__ void __launch_bounds__(CM_THREADS) k_cholmod(double *S, int n, int ld, double *E, double *work)
{
    __shared__ double dred[CM_THREADS];
    __shared__ int ired[CM_THREADS];
    __shared__ double sh_T[9], sh_L[6], sh_Li[9];
    __shared__ int sh_fail;
    double *diag = work;          // n
    double *orig = work + n;      // 3 n
    double *C = work + 4 * n;     // n
    const int tid = threadIdx.x;
    // xi = max |offdiag|, gamma = max |diag| over the symmetric matrix (lower read)
    double xi = 0.0, gam = 0.0;
    for (long long e = tid; e < (long long)n * n; e += CM_THREADS) {
        const int r = (int)(e / n), k = (int)(e % n);
        if (r == k) {
            gam = fmax(gam, fabs(S[(size_t)r * ld + r]));
        } else {
            const int hi = r > k ? r : k, lo = r > k ? k : r;
            xi = fmax(xi, fabs(S[(size_t)hi * ld + lo]));
        }
    }
    xi = block_max(xi, dred);
    gam = block_max(gam, dred);
    const double delta = 1e-15 * fmax(xi + gam, 1.0);
    double beta = fmax(gam, 1e-15);
    beta = fmax(beta, xi / sqrt((double)(n * n - 1)));
    beta = sqrt(beta);
    for (int r = tid; r < n; r += CM_THREADS) diag[r] = S[(size_t)r * ld + r];
    __syncthreads();
    const int nb = n / 3;
    for (int j = 0; j < nb; ++j) {
        for (int e = tid; e < (n - 3 * j) * 3; e += CM_THREADS) {
            const int r = 3 * j + e / 3, v = e % 3;
            orig[(size_t)r * 3 + v] = S[(size_t)r * ld + 3 * j + v];
        }
        __syncthreads();
        if (tid < 9) {
            const int u = tid / 3, v = tid % 3;
            const int ru = 3 * j + u, rv = 3 * j + v;
            double sum = v > u ? S[(size_t)rv * ld + ru] : S[(size_t)ru * ld + rv];
            const double *lu = S + (size_t)ru * ld, *lv = S + (size_t)rv * ld;
            for (int k = 0; k < j; ++k)
                sum -= (lu[3 * k] * lv[3 * k] + lu[3 * k + 1] * lv[3 * k + 1] + lu[3 * k + 2] * lv[3 * k + 2]);
            sh_T[tid] = sum;
        }
        __syncthreads();
        if (tid == 0) {
            const double *Tm = sh_T;
            int fail = 0;
            const double p0 = Tm[0];
            const double p1 = Tm[4] - Tm[3] * Tm[3] / Tm[0];
            const double t1 = -Tm[8] * Tm[3] * Tm[3], t2 = 2 * Tm[7] * Tm[3] * Tm[6],
                         t3 = -Tm[4] * Tm[6] * Tm[6];
            const double t4 = Tm[0] * (Tm[4] * Tm[8] - Tm[7] * Tm[7]),
                         t5 = -Tm[3] * Tm[3] + Tm[0] * Tm[4];
            const double p2 = (t1 + t2 + t3 + t4) / t5;
            if (!isfinite(p0) || p0 <= 0 || !isfinite(p1) || p1 <= 0 || !isfinite(p2) || p2 <= 0) fail = 1;
            if (!fail) {
                double *L = sh_L;
                L[0] = sqrt(p0);
                L[1] = Tm[3] / sqrt(Tm[0]);
                L[2] = sqrt(p1);
                L[3] = Tm[6] / sqrt(Tm[0]);
                L[4] = sqrt(Tm[0] / (Tm[0] * Tm[4] - Tm[3] * Tm[3])) * (Tm[7] - Tm[3] * Tm[6] / Tm[0]);
                L[5] = sqrt(p2);
                if (!isfinite(L[1]) || !isfinite(L[3]) || !isfinite(L[4])) fail = 1;
                double *Li = sh_Li;
                Li[0] = 1 / L[0]; Li[1] = 0; Li[2] = 0;
                Li[3] = -L[1] / (L[0] * L[2]); Li[4] = 1 / L[2]; Li[5] = 0;
                Li[6] = (L[1] * L[4] - L[2] * L[3]) / (L[0] * L[2] * L[5]);
                Li[7] = -L[4] / (L[2] * L[5]); Li[8] = 1 / L[5];
            }
            sh_fail = fail;
        }
        __syncthreads();
        int fail = sh_fail;
        if (!fail) {
            // write the diagonal block, then the blocks below: T_ij then L_ij = T_ij Li^T
            if (tid == 0) {
                double *dd = S + (size_t)(3 * j) * ld + 3 * j;
                dd[0] = sh_L[0]; dd[1] = 0; dd[2] = 0;
                dd[ld] = sh_L[1]; dd[ld + 1] = sh_L[2]; dd[ld + 2] = 0;
                dd[2 * ld] = sh_L[3]; dd[2 * ld + 1] = sh_L[4]; dd[2 * ld + 2] = sh_L[5];
            }
            __syncthreads();
            int big = 0;
            for (int blk = j + 1 + tid; blk < nb; blk += CM_THREADS) {
                double Tij[9];
                for (int u = 0; u < 3; ++u)
                    for (int v = 0; v < 3; ++v) {
                        const int ri = 3 * blk + u, rj = 3 * j + v;
                        double sum = S[(size_t)ri * ld + rj];
                        const double *lu = S + (size_t)ri * ld, *lv = S + (size_t)rj * ld;
                        for (int k = 0; k < j; ++k)
                            sum -= (lu[3 * k] * lv[3 * k] + lu[3 * k + 1] * lv[3 * k + 1] +
                                    lu[3 * k + 2] * lv[3 * k + 2]);
                        Tij[u * 3 + v] = sum;
                    }
                for (int u = 0; u < 3; ++u)
                    for (int v = 0; v < 3; ++v) {
                        const double val = (Tij[u * 3] * sh_Li[v * 3] + Tij[u * 3 + 1] * sh_Li[v * 3 + 1] +
                                            Tij[u * 3 + 2] * sh_Li[v * 3 + 2]);
                        S[(size_t)(3 * blk + u) * ld + 3 * j + v] = val;
                        S[(size_t)(3 * j + v) * ld + 3 * blk + u] = 0.0;
                        if (val > beta) big = 1;
                    }
            }
            fail = block_or(big, ired);
        }
        if (!fail) continue;
        // restore column block j and redo its columns one at a time
        for (int e = tid; e < (n - 3 * j) * 3; e += CM_THREADS) {
            const int r = 3 * j + e / 3, v = e % 3;
            S[(size_t)r * ld + 3 * j + v] = orig[(size_t)r * 3 + v];
        }
        __syncthreads();
        for (int col = 0; col < 3; ++col) {
            const int x = 3 * j + col;
            if (tid == 0) {
                double sum = S[(size_t)x * ld + x];
                for (int k = 0; k < x; ++k) {
                    const double l = S[(size_t)x * ld + k];
                    sum -= l * l;
                }
                sum = fabs(sum);
                S[(size_t)x * ld + x] = sqrt(fmax(sum, delta));
            }
            __syncthreads();
            const double lxx = S[(size_t)x * ld + x];
            int big = 0;
            for (int i = x + 1 + tid; i < n; i += CM_THREADS) {
                double c = S[(size_t)i * ld + x];
                for (int k = 0; k < x; ++k) c = c - (S[(size_t)i * ld + k] * S[(size_t)x * ld + k]);
                C[i] = c;
                const double l = c / lxx;
                S[(size_t)i * ld + x] = l;
                S[(size_t)x * ld + i] = 0.0;
                if (l > beta) big = 1;
            }
            big = block_or(big, ired);
            if (big) {
                double th = 0.0;
                for (int i = x + 1 + tid; i < n; i += CM_THREADS) th = fmax(th, fabs(C[i]));
                th = block_max(th, dred);
                const double nl = th / beta;
                if (tid == 0) S[(size_t)x * ld + x] = nl;
                for (int i = x + 1 + tid; i < n; i += CM_THREADS) S[(size_t)i * ld + x] = C[i] / nl;
            }
            __syncthreads();
        }
    }
    __syncthreads();
    for (int i = tid; i < n; i += CM_THREADS) {
        double sum = 0.0;
        for (int k = 0; k <= i; ++k) sum += S[(size_t)i * ld + k] * S[(size_t)i * ld + k];
        E[i] = sum - diag[i];
    }
}

void launch_cholmod(double *S, int n, int ld, double *E, double *work, cudaStream_t s)
{
    k_cholmod<<<1, CM_THREADS, 0, s>>>(S, n, ld, E, work); note_launch(1);
}

}  // namespace psba

// Dense FP64 reduced-camera solve on sm_103a.
//
// S (Np x Np, lower triangle, Np a multiple of TILE) is factored S = L L^T
// by one cooperative persistent kernel over TILE x TILE lower tiles.  CTA 0
// (the panel) walks the diagonal: it applies the last update to each
// diagonal tile, factors it (cta_potrf, with the forward solve of rhs carried
// along) and forms the sub-diagonal tile below it, which it keeps for the
// next step.  The other CTAs (helpers) accumulate every other update
// (left-looking) and solve the remaining tiles against the diagonal
// inverses, in a fixed dependency order; waits are bounded spins on per-task
// flags in global memory (acquire/release).  After the factor, the back
// solve L^T x = y runs on a thread-block cluster (k_tri_cluster; k_tri_solve,
// one CTA, when PSBA_TRI_CLUSTER is 0).  On request one step of iterative
// refinement follows: r = b - S x in FP64 against a copy of S taken before
// the factor (k_refine_residual), then both triangular solves of r with the
// factor, added into x (the same kernels with their forward part on).
//
// This replaces the reference's explicit inverse (SPD_inv.cl: 3x3-block
// Cholesky chain, kern_trigMat_inv, kern_trigMat_mul, then matVec_mul) with
// two triangular solves.  The failure test is the reference's: a non-positive
// or non-finite pivot (SPD_inv.cl:66-107) sets status 1; every task still
// raises its flag, so nothing waits forever.  A spin that runs out of its
// iteration budget sets status 2 and the kernel completes.
#include <cfloat>
#include <cooperative_groups.h>
#include <mutex>
#include <vector>

#include "psba_internal.h"

namespace psba {

namespace cg = cooperative_groups;

constexpr int T = TILE;
constexpr int TT = TILE * TILE;
// Launch shape (compile-time tuning knobs): threads per CTA, update steps
// staged per batch, and a cap on CTAs per SM (0: as many as fit).
#ifndef PSBA_CHOL_THREADS
#define PSBA_CHOL_THREADS 256
#endif
#ifndef PSBA_CHOL_BJ
#define PSBA_CHOL_BJ 8
#endif
#ifndef PSBA_TRI_CLUSTER
#define PSBA_TRI_CLUSTER 1  // triangular solves on a cluster of CTAs (else one CTA)
#endif
#ifndef PSBA_CHOL_PER_SM
#define PSBA_CHOL_PER_SM 1  // the panel's FP64 chain runs alone on its SM
#endif
constexpr int CF_THREADS = PSBA_CHOL_THREADS;
// Polls per wait (each poll an acquire load and a 64 ns sleep; the default,
// 2^22, is ~0.5 s) come from the launch: a handle can shorten the bound
// (psba_set_wait_limit).  Thread 0 of each CTA stores it here at entry.
__shared__ long long s_spin_limit;
constexpr int BJ = PSBA_CHOL_BJ;             // update steps staged per batch in a tile task
static_assert(BJ >= 2, "the diagonal factor reuses two staging tiles");


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
        const long long limit = s_spin_limit;
        for (long long it = 0; it < limit; ++it) {
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

// ---------------------------------------------------------------------------
// Diagonal-tile factor.  GB300 issues one FP64 warp instruction per ~64
// cycles however many lanes are active, and an FP64 result is ready ~64
// cycles after issue, so the factor of a 16 x 16 tile is bound by its chain
// of dependent pivots (d_s, then 1/sqrt(d_s)) and by how much latency the
// rest adds per column.  The plan below keeps everything but the pivot chain
// off warp 0 and gives every other thread a fixed, index-free role, in
// T + 1 phases separated by one barrier each (named barrier 1, the seven warps
// with a role):
//   warp 0    phase s: d_s = a[s][s] - (a[s][s-1] / L_{s-1,s-1})^2 (the last
//             update of the pivot, one column ahead of the others), 1/L_ss
//             and 1/d_s.
//   trailing  (warps 2, 3, 6, 7) own the entries a[r][j], 1 <= j <= r, and
//             b[r] (as column T) in registers.  Phase s applies column s-1:
//             a[r][j] -= a[r][s-1] a[j][s-1] / d_{s-1}; an entry is published
//             to shared memory in the phase it becomes final, and its L
//             value (a[r][j] / L_jj, y_r = b_r / L_rr) written in the next.
//   inverse   (warps 1, 5) build X = L^-1 one column behind L: entry (i, c)
//             takes X[i][c] -= L[i][k] X[k][c] in phase k + 2, c <= k < i,
//             and X[i][c] /= L_ii in its last phase; entries are dealt to
//             threads by interval colouring, so a thread has one at a time.
//   warp 4    shares warp 0's sub-partition and takes no part in the phases
//             (the panel gives it the step's stores and fetches).
// Each role runs the same short instruction sequence in every lane (operands
// picked by selects), so a trailing warp issues two FP64 instructions per
// phase.  The roles run alongside the chain but still slow it (the chain
// alone: ~710 cycles per column; all roles: ~840); this placement of the
// roles and the published 1/d_s measured 7% faster than trailing on warps
// 1, 2, 3, 5 computing 1/d_s themselves.  The plan is built at compile time
// and copied to shared memory once per launch (divergent reads of constant
// memory serialise).

enum : unsigned char { PF_NONE = 0, PF_OFF, PF_DIAG, PF_D11, PF_B, PF_COL0, PF_B0 };
constexpr int PF_TRAIL = 128, PF_INV = 64, PF_INV_MAX = 16;
constexpr int PF_BCOL = T;  // b rides along as column T

struct PfEntry {
    unsigned char kind, r, j;
};
struct PfPlan {
    PfEntry tr[PF_TRAIL][2];
    unsigned char inv_i[PF_INV][PF_INV_MAX], inv_c[PF_INV][PF_INV_MAX], inv_n[PF_INV];
};

// last phase in which an entry does work (update, publication or L value)
__host__ __device__ constexpr int pf_last_busy(const PfEntry &e)
{
    return e.kind == PF_OFF ? e.j + 1 : e.kind == PF_DIAG ? e.j + 1 : e.kind == PF_D11 ? 2 : e.kind == PF_B ? e.r + 1 : 1;
}

constexpr PfPlan make_pf_plan()
{
    PfPlan p{};
    PfEntry ents[T * (T + 1) / 2 + T + 1] = {};
    int n = 0;
    for (int j = 1; j < T; ++j)
        for (int r = j + 1; r < T; ++r) ents[n++] = PfEntry{PF_OFF, (unsigned char)r, (unsigned char)j};
    for (int j = 2; j < T; ++j) ents[n++] = PfEntry{PF_DIAG, (unsigned char)j, (unsigned char)j};
    ents[n++] = PfEntry{PF_D11, 1, 1};
    for (int r = 1; r < T; ++r) ents[n++] = PfEntry{PF_B, (unsigned char)r, (unsigned char)PF_BCOL};
    for (int r = 0; r < T; ++r) ents[n++] = PfEntry{PF_COL0, (unsigned char)r, 0};
    ents[n++] = PfEntry{PF_B0, 0, (unsigned char)PF_BCOL};
    // stable sort by last busy phase, latest first
    for (int a = 1; a < n; ++a) {
        const PfEntry v = ents[a];
        int b = a;
        while (b > 0 && pf_last_busy(ents[b - 1]) < pf_last_busy(v)) {
            ents[b] = ents[b - 1];
            --b;
        }
        ents[b] = v;
    }
    for (int u = 0; u < PF_TRAIL; ++u) {
        p.tr[u][0] = ents[u];
        p.tr[u][1] = PfEntry{PF_NONE, 0, 0};
    }
    for (int q = PF_TRAIL; q < n; ++q) p.tr[q - PF_TRAIL][1] = ents[q];
    // inverse entries (i, c), i > c, busy in phases [c + 2, i + 1]: generated
    // by start, each goes to the first thread whose previous entry has ended
    for (int v = 0; v < PF_INV; ++v) p.inv_n[v] = 0;
    for (int c = 0; c < T; ++c)
        for (int i = c + 1; i < T; ++i)
            for (int v = 0; v < PF_INV; ++v) {
                const int m = p.inv_n[v];
                if (m < PF_INV_MAX && (m == 0 || p.inv_i[v][m - 1] + 1 < c + 2)) {
                    p.inv_i[v][m] = (unsigned char)i;
                    p.inv_c[v][m] = (unsigned char)c;
                    p.inv_n[v] = (unsigned char)(m + 1);
                    break;
                }
            }
    return p;
}

constexpr PfPlan kPfPlan = make_pf_plan();

constexpr bool pf_plan_ok()
{
    // second entries are only busy in phases 1-2; every inverse entry placed
    int placed = 0;
    for (int u = 0; u < PF_TRAIL; ++u)
        if (kPfPlan.tr[u][1].kind != PF_NONE && pf_last_busy(kPfPlan.tr[u][1]) > 2) return false;
    for (int v = 0; v < PF_INV; ++v) placed += kPfPlan.inv_n[v];
    return placed == T * (T - 1) / 2;
}
static_assert(pf_plan_ok(), "diagonal-tile factor plan");

__constant__ PfPlan c_pf = kPfPlan;

// the factor plan into shared memory (once per launch)
__device__ void load_pf_plan(PfPlan &dst)
{
    const unsigned char *src = reinterpret_cast<const unsigned char *>(&c_pf);
    unsigned char *d = reinterpret_cast<unsigned char *>(&dst);
    for (int i = threadIdx.x; i < (int)sizeof(PfPlan); i += blockDim.x) d[i] = src[i];
    __syncthreads();
}

// The factor's workspace: one shared block of doubles, so that every access
// is an offset from one base (fixed per entry, plus a phase constant once
// the phase loop is unrolled).
constexpr int PW_ROW = T + 1;            // padded row
constexpr int PW_A = 0;                  // the tile (published entries, pivots)
constexpr int PW_L = T * PW_ROW;         // the factor L
constexpr int PW_LINV = 2 * T * PW_ROW;  // its inverse
constexpr int PW_BW = 3 * T * PW_ROW;    // b being reduced
constexpr int PW_INVD = PW_BW + T;       // 1 / L_kk = d_k^-1/2 (final pass)
constexpr int PW_Y = PW_BW + 2 * T;      // y = L^-1 b
constexpr int PW_B = PW_BW + 3 * T;      // b (input)
constexpr int PW_INV2 = PW_BW + 4 * T;   // 1 / d_k (warp 0 publishes it)
constexpr int PW_ASQ = PW_BW + 5 * T;    // a_k,k-1^2 (published with a_k,k-1)
constexpr int PW_SIZE = PW_BW + 6 * T;

// One entry of a trailing thread, decoded once per factor into offsets: the
// entry's row (xo), the other operand of its update (oo: row j of the tile,
// or b), the source of its L value when that is not the entry itself (lo),
// the pivot inverse it divides by (qo), where it is published (po) and where
// its L value goes (dofs), its last update phase (0: none) and the phase its
// L value is due.
struct PfSlot {
    int xo, oo, lo, qo, po, dofs, last, due;
    bool lself;
    int sqo;  // entry (j + 1, j): where its square goes when final, else -1
};

__device__ __forceinline__ PfSlot pf_slot(const PfEntry &e)
{
    const int r = e.r, j = e.j;
    switch (e.kind) {
    case PF_OFF:
        return PfSlot{r * PW_ROW, j * PW_ROW, 0, PW_INV2 + j, r * PW_ROW + j, PW_L + r * PW_ROW + j, j, j + 1, true,
                      r == j + 1 ? PW_ASQ + r : -1};
    case PF_DIAG:  // d_j is left in a[j][j] by warp 0; its M value (1) is not read
        return PfSlot{j * PW_ROW, j * PW_ROW, j * PW_ROW + j, PW_INV2 + j, j * PW_ROW + j, PW_L + j * PW_ROW + j, j - 1,
                      j + 1, false, -1};
    case PF_D11:
        return PfSlot{PW_ROW, PW_ROW, PW_ROW + 1, PW_INV2 + 1, 0, PW_L + PW_ROW + 1, 0, 2, false, -1};
    case PF_B:  // its M value is not read: the final pass forms y from the entry
        return PfSlot{r * PW_ROW, PW_BW, 0, PW_INV2 + r, PW_BW + r, PW_Y + r, r, r + 1, true, -1};
    case PF_COL0:
        return PfSlot{r * PW_ROW, 0, r * PW_ROW, PW_INV2, 0, PW_L + r * PW_ROW, 0, 1, false, -1};
    case PF_B0:
        return PfSlot{0, PW_BW, PW_BW, PW_INV2, 0, PW_Y, 0, 1, false, -1};
    default:
        return PfSlot{0, 0, 0, 0, 0, 0, 0, 0, true, -1};
    }
}

// Phase s >= 1 of one entry: the update v -= a[r][k] (other[k] / d_k),
// k = s - 1, or its L value, as two FP64 instructions whatever the entry
// does (loads unconditional and in bounds, operands picked by selects).
template <int S>
__device__ __forceinline__ void pf_step(const PfSlot &q, double &v, double ik2, double *W)
{
    constexpr int k = S - 1;
    const bool upd = S <= q.last, lval = S == q.due;
    const double xk = W[q.xo + k];
    const double ok = W[q.oo + k];
    const double lraw = W[q.lo];
    const double qi = W[q.qo];
    const double lv = q.lself ? v : lraw;
    const double pa = upd ? ok : lval ? lv : 0.0;
    const double qa = upd ? ik2 : lval ? qi : 0.0;
    const double t = pa * qa;
    const double xs = upd ? xk : 0.0;  // a select of the value; the sign rides on the FMA
    v = fma(-xs, t, v);
    if (upd && S == q.last) {
        W[q.po] = v;
        if (q.sqo >= 0) W[q.sqo] = v * v;
    }
    if (lval) W[q.dofs] = t;
}

// Phase S of the whole CTA (see the plan above).
// The phases synchronise the seven warps with a role (named barrier 1); warp
// 4 joins the CTA only at the factor's start and end.
__device__ __forceinline__ void pf_barrier() { asm volatile("bar.sync 1, %0;" ::"n"(CF_THREADS - 32) : "memory"); }

template <int S>
__device__ __forceinline__ void pf_phase(double *W, int warp, int u, int vi, int wlast, const PfPlan &pf,
                                         const PfSlot &q0, const PfSlot &q1, double &v0, double &v1,
                                         double &inv_prev, double &w, int &wi, int n_inv, int &ci, int &cc)
{
    if (warp == 0) {
        // the last phase has no pivot: 1 / sqrt(d_j) for the final pass
        if (S == T && threadIdx.x < T) W[PW_INVD + threadIdx.x] = rsqrt(W[PW_A + threadIdx.x * PW_ROW + threadIdx.x]);
        // the pivot chain: d_S = a_SS - a_S,S-1^2 / d_S-1 and 1 / d_S, no root
        if (S < T && threadIdx.x == 0) {
            double d = W[PW_A + S * PW_ROW + S];
            if (S > 0) {
                double asq;
                if (S == 1) {
                    const double a = W[PW_A + PW_ROW];
                    asq = a * a;
                } else {
                    asq = W[PW_ASQ + S];
                }
                d = fma(-asq, inv_prev, d);
                W[PW_A + S * PW_ROW + S] = d;
            }
            inv_prev = rcp_fast(d);
            W[PW_INV2 + S] = inv_prev;
        }
    } else if (u >= 0) {
        // a trailing warp whose entries are all done skips the phase (its
        // FP64 instructions would hold up the pipe that the chain shares)
        if (S >= 1 && S <= wlast) {
            const double ik2 = W[PW_INV2 + (S >= 1 ? S - 1 : 0)];
            pf_step<S>(q0, v0, ik2, W);
            if (S <= 2) pf_step<S>(q1, v1, ik2, W);
        }
    } else if (vi >= 0) {
        if (S >= 2) {
            constexpr int k = S >= 2 ? S - 2 : 0;
            if (S > ci + 1 && wi + 1 < n_inv) {  // entries are disjoint in time: at most one step
                ++wi;
                ci = pf.inv_i[vi][wi];
                cc = pf.inv_c[vi][wi];
                w = 0.0;
            }
            if (S >= cc + 2 && S <= ci + 1) {
                w = fma(-W[PW_L + ci * PW_ROW + k], W[PW_LINV + k * PW_ROW + cc], w);
                if (S == ci + 1) W[PW_LINV + ci * PW_ROW + cc] = w;
            }
        }
    }
    pf_barrier();
}

template <int S>
__device__ __forceinline__ void pf_phases(double *W, int warp, int u, int vi, int wlast, const PfPlan &pf,
                                          const PfSlot &q0, const PfSlot &q1, double &v0, double &v1,
                                          double &inv_prev, double &w, int &wi, int n_inv, int &ci, int &cc)
{
    if constexpr (S <= T) {
        pf_phase<S>(W, warp, u, vi, wlast, pf, q0, q1, v0, v1, inv_prev, w, wi, n_inv, ci, cc);
        pf_phases<S + 1>(W, warp, u, vi, wlast, pf, q0, q1, v0, v1, inv_prev, w, wi, n_inv, ci, cc);
    }
}

// All threads (CF_THREADS == 256): Cholesky of the lower triangle of the
// tile W[PW_A..] into the lower triangle of W[PW_L..], its inverse into the
// lower triangle of W[PW_LINV..] (the upper triangles are left as they were:
// nothing reads them), 1 / L_kk into W[PW_INVD..] and y = L^-1 b (b in
// W[PW_B..]) into W[PW_Y..], following the plan pf (in shared memory).
// Returns false on a non-positive or non-finite pivot (checked once at the
// end: a bad pivot only produces non-finite values downstream).
// warp 4's work during the factor: none
struct NoSide {
    __device__ __forceinline__ void run(const int *) {}
};

template <typename Side = NoSide>
__device__ bool cta_potrf(double *W, const PfPlan &pf, Side &&side = Side())
{
    static_assert(CF_THREADS == 256, "the factor plan is laid out for eight warps");
    __shared__ int bad, fdone;
    const int tid = threadIdx.x, warp = tid >> 5;
    if (tid < T) W[PW_BW + tid] = W[PW_B + tid];
    if (tid == 0) {
        bad = 0;
        fdone = 0;
    }
    const int u = (warp == 2 || warp == 3) ? tid - 64 : (warp == 6 || warp == 7) ? tid - 128 : -1;
    const int vi = warp == 1 ? tid - 32 : warp == 5 ? tid - 128 : -1;
    PfSlot q0 = pf_slot(PfEntry{PF_NONE, 0, 0}), q1 = q0;
    double v0 = 0.0, v1 = 0.0;
    int wlast = 0;  // a trailing warp's last busy phase
    if (u >= 0) {
        const PfEntry e0 = pf.tr[u][0], e1 = pf.tr[u][1];
        q0 = pf_slot(e0);
        q1 = pf_slot(e1);
        v0 = W[e0.j == PF_BCOL ? PW_B + e0.r : PW_A + e0.r * PW_ROW + e0.j];
        v1 = W[e1.j == PF_BCOL ? PW_B + e1.r : PW_A + e1.r * PW_ROW + e1.j];
        const int busy = e0.kind == PF_NONE ? 0 : pf_last_busy(e0);
        wlast = __reduce_max_sync(0xffffffffu, max(busy, e1.kind == PF_NONE ? 0 : pf_last_busy(e1)));
    }
    // inverse threads: the current entry (ci, cc) in registers, the list read
    // only when an entry is done
    const int n_inv = vi >= 0 ? pf.inv_n[vi] : 0;
    int wi = 0, ci = -2, cc = T;
    if (n_inv > 0) {
        ci = pf.inv_i[vi][0];
        cc = pf.inv_c[vi][0];
    }
    __syncthreads();
    double inv_prev = 0.0, w = 0.0;
    if (warp == 4) {
        side.run(&fdone);
    } else {
        // after the CTA barrier above: until then the panel's side warp may
        // still be storing the previous tile's inverse from this workspace
        if (tid < T) W[PW_LINV + tid * PW_ROW + tid] = 1.0;  // M^-1 has a unit diagonal
        pf_phases<0>(W, warp, u, vi, wlast, pf, q0, q1, v0, v1, inv_prev, w, wi, n_inv, ci, cc);
        // the phases leave the pivots d_j on the diagonal, the final entries
        // a_rj below it, M = a_rj / d_j in W[PW_L..], M^-1 in W[PW_LINV..]
        // and 1 / sqrt(d_j) in W[PW_INVD..]; with D^1/2 = diag(sqrt(d_j)):
        // L = a D^-1/2, L^-1 = D^-1/2 M^-1, y = D^-1/2 z
        static_assert(T == 16, "entry (r, j) = (e >> 4, e & 15)");
        const int rt = tid < 128 ? tid : tid - 32;  // 0 .. 223 over the seven warps with a role
        for (int e = rt; e < T * T; e += CF_THREADS - 32) {
            const int r = e >> 4, j = e & (T - 1);
            if (j <= r) {
                W[PW_L + r * PW_ROW + j] = W[PW_A + r * PW_ROW + j] * W[PW_INVD + j];
                W[PW_LINV + r * PW_ROW + j] *= W[PW_INVD + r];
            }
            if (e < T) W[PW_Y + e] = W[PW_BW + e] * W[PW_INVD + e];
        }
        if (tid == 0) *(volatile int *)&fdone = 1;
    }
    if (tid < T) {
        const double d = W[PW_A + tid * PW_ROW + tid];
        if (!(d >= DBL_MIN) || !isfinite(d)) bad = 1;  // the reciprocal flushes subnormals
    }
    __syncthreads();
    return bad == 0;
}

// The single-CTA back solve over the factor (S lower = L, Linv = diagonal
// tile inverses) with the right-hand side in shared memory.  A block step is
// the 16 x 16 product with the diagonal inverse, then the update of the other
// blocks, one column of it per thread, reading one row panel of L with
// independent loads; it is bound by the SM's FP64 rate (N^2 / 2
// multiply-adds on one SM).  The diagonal product is spread over 256 threads
// (one product each, summed by a fixed shuffle tree over 16 lanes), and the
// values a thread needs for the next block step (its Linv entry, its 16
// panel values) are loaded while the current one runs.

// One lane of the 16 x 16 diagonal product: 16 lanes hold the products of one
// output, summed in a fixed order.
__device__ __forceinline__ double half_warp_sum(double p)
{
#pragma unroll
    for (int off = T / 2; off > 0; off >>= 1) p += __shfl_xor_sync(0xffffffffu, p, off);
    return p;
}

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
// then y_I -= L_KI^T x_K for I < K, reading rows K*T..K*T+T-1 of L); acc: x
// += the solution instead.
__device__ void cta_back(int Np, int nb, const double *__restrict__ S, const double *__restrict__ Linv,
                         double *ys, double *xs, double *__restrict__ x, bool acc, float2 *__restrict__ x2)
{
    const int tid = threadIdx.x, nthr = blockDim.x;
    const int dc = tid / T, dk = tid % T;  // diagonal product: output column, term
    auto load_diag = [&](int K) {
        return (tid < TT && dk >= dc) ? __ldcg(Linv + (size_t)K * TT + dk * T + dc) : 0.0;
    };
    auto load_panel = [&](int K, double (&v)[T]) {
        if (tid < K * T) {
            const double *base = S + (size_t)(K * T) * Np + tid;
#pragma unroll
            for (int c = 0; c < T; ++c) v[c] = __ldcg(base + (size_t)c * Np);
        }
    };
    double curL = load_diag(nb - 1), curS[T] = {}, nxtS[T] = {};
    load_panel(nb - 1, curS);
    for (int K = nb - 1; K >= 0; --K) {
        double nxtL = 0.0;
        if (K > 0) {
            nxtL = load_diag(K - 1);
            load_panel(K - 1, nxtS);
        }
        if (tid < TT) {
            const double v = half_warp_sum(curL * ys[K * T + dk]);
            if (dk == 0) {
                xs[dc] = v;
                const double xv = acc ? x[K * T + dc] + v : v;
                x[K * T + dc] = xv;
                if (x2) x2[K * T + dc] = split2f(xv);
            }
        }
        __syncthreads();
        if (tid < K * T) {
            double s = 0.0;
#pragma unroll
            for (int c = 0; c < T; ++c) s = fma(curS[c], xs[c], s);
            ys[tid] -= s;
        }
        for (int col = tid + nthr; col < K * T; col += nthr) {  // columns beyond the prefetched one
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
        curL = nxtL;
#pragma unroll
        for (int c = 0; c < T; ++c) curS[c] = nxtS[c];
    }
}

// Dealt-out tile products.  A tile operation costs the largest number of
// FP64 instructions any thread of a warp runs, so the products below are
// spread evenly over the CTA.

// a[r][c] -= sum_k L[r][k] L[c][k] for c <= r and, when WITH_B,
// b[r] -= sum_k L[r][k] y[k]: the NE x T products (element, k) are cut into
// consecutive runs of PER, one per thread; a run spans at most NACC
// elements, whose partial sums go to part[NACC t ...].  Each element then
// subtracts its partial sums in k order.  The accumulator and operands of a
// product are picked by selects, so a warp issues one FMA per product.
__device__ __forceinline__ void tri_of(int e, int &r, int &c)
{
    r = (int)((sqrtf(8.0f * (float)e + 1.0f) - 1.0f) * 0.5f);
    while ((r + 1) * (r + 2) / 2 <= e) ++r;
    while (r * (r + 1) / 2 > e) --r;
    c = e - r * (r + 1) / 2;
}

template <bool WITH_B, int NT = CF_THREADS>
struct LowerUpdate {
    static constexpr int NTRI = T * (T + 1) / 2;
    static constexpr int NE = NTRI + (WITH_B ? T : 0);
    static constexpr int PER = (NE * T + NT - 1) / NT;
    static constexpr int NACC = (T - 1 + PER + T - 1) / T;  // elements one run can touch
    static constexpr int PART = NACC * NT;                  // doubles of partial sums
};

// NT == CF_THREADS: the whole CTA, CTA barriers.  NT == CF_THREADS - 32: every
// warp but warp 4 (the panel's), on named barrier 1.
template <bool WITH_B, int NT = CF_THREADS>
__device__ void update_lower(double (*a)[T + 1], const double (*L)[T + 1], double *b, const double *y, double *part)
{
    static_assert(NT == CF_THREADS || NT == CF_THREADS - 32, "whole CTA or all warps but warp 4");
    using U = LowerUpdate<WITH_B, NT>;
    constexpr int NTRI = U::NTRI, NE = U::NE, PER = U::PER, NACC = U::NACC;
    auto sync = [] {
        if (NT == CF_THREADS) __syncthreads();
        else asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
    };
    const int tid = NT == CF_THREADS ? (int)threadIdx.x : (int)threadIdx.x - ((int)threadIdx.x >= 160 ? 32 : 0);
    const int f0 = tid * PER, e0 = f0 / T;
    const double *xs[NACC], *ys[NACC];
    double p[NACC];
#pragma unroll
    for (int j = 0; j < NACC; ++j) {
        const int ej = min(e0 + j, NE - 1);
        int r, c;
        if (ej < NTRI) {
            tri_of(ej, r, c);
            xs[j] = L[r];
            ys[j] = L[c];
        } else {
            xs[j] = L[ej - NTRI];
            ys[j] = y;
        }
        p[j] = 0.0;
    }
#pragma unroll
    for (int i = 0; i < PER; ++i) {
        const int f = f0 + i;
        const int k = f % T, idx = f / T - e0;
        const bool valid = f < NE * T;
        const double *xp = xs[0], *yp = ys[0];
        double acc = p[0];
#pragma unroll
        for (int j = 1; j < NACC; ++j) {
            xp = idx == j ? xs[j] : xp;
            yp = idx == j ? ys[j] : yp;
            acc = idx == j ? p[j] : acc;
        }
        const double v = fma(valid ? xp[k] : 0.0, valid ? yp[k] : 0.0, acc);
#pragma unroll
        for (int j = 0; j < NACC; ++j) p[j] = idx == j ? v : p[j];
    }
#pragma unroll
    for (int j = 0; j < NACC; ++j) part[NACC * tid + j] = p[j];
    sync();
    for (int e2 = tid; e2 < NE; e2 += NT) {
        const int tlo = (e2 * T) / PER, thi = (e2 * T + T - 1) / PER;
        int r = 0, c = 0;
        if (e2 < NTRI) tri_of(e2, r, c);
        double v = e2 < NTRI ? a[r][c] : b[e2 - NTRI];
        for (int t = tlo; t <= thi; ++t) v -= part[NACC * t + (e2 - (t * PER) / T)];
        if (e2 < NTRI) a[r][c] = v;
        else b[e2 - NTRI] = v;
    }
    sync();
}

// The panel's last update of the diagonal tile and of b, a -= L L^T and
// b -= L y over the lower triangle, one output per thread (152 outputs, 224
// threads on named barrier 1): sixteen multiply-adds in two interleaved
// chains of eight, then one subtraction.  One pass, where update_lower's
// even deal of the products needs partial sums, a barrier and a second pass.
__device__ void update_lower_panel(double (*a)[T + 1], const double (*L)[T + 1], double *b, const double *y)
{
    constexpr int NT = CF_THREADS - 32, NTRI = T * (T + 1) / 2, NE = NTRI + T;
    static_assert(NE <= NT, "one output per thread");
    const int tid = (int)threadIdx.x - ((int)threadIdx.x >= 160 ? 32 : 0);
    if (tid < NE) {
        int r = 0, c = 0;
        const double *xr, *yr;
        double *dst;
        if (tid < NTRI) {
            tri_of(tid, r, c);
            xr = L[r];
            yr = L[c];
            dst = &a[r][c];
        } else {
            xr = L[tid - NTRI];
            yr = y;
            dst = b + (tid - NTRI);
        }
        double s0 = 0.0, s1 = 0.0;
#pragma unroll
        for (int k = 0; k < T; k += 2) {
            s0 = fma(xr[k], yr[k], s0);
            s1 = fma(xr[k + 1], yr[k + 1], s1);
        }
        *dst -= s0 + s1;
    }
    asm volatile("bar.sync 1, %0;" ::"n"(NT) : "memory");
}

// out = A Linv^T restricted to the lower triangle of Linv (out[r][c] =
// sum_{k <= c} A[r][k] Linv[c][k]): columns c and T-1-c of a row go to one
// thread, T + 1 products each.
__device__ void tile_trsm(double (*out)[T + 1], const double (*A)[T + 1], const double (*Li)[T + 1])
{
    for (int p = threadIdx.x; p < TT / 2; p += CF_THREADS) {
        const int r = p / (T / 2), c0 = p % (T / 2), c1 = T - 1 - c0;
        double s0 = 0.0, s1 = 0.0;
#pragma unroll
        for (int i = 0; i < T + 1; ++i) {
            const bool first = i <= c0;
            const int c = first ? c0 : c1, k = first ? i : i - c0 - 1;
            const double v = fma(A[r][k], Li[c][k], first ? s0 : s1);
            s0 = first ? v : s0;
            s1 = first ? s1 : v;
        }
        out[r][c0] = s0;
        out[r][c1] = s1;
    }
}

__device__ __forceinline__ void store_tile(double *S, int Np, int I, int K, const double (*t)[T + 1])
{
    for (int e = threadIdx.x; e < TT; e += CF_THREADS) S[(size_t)(I * T + e / T) * Np + K * T + e % T] = t[e / T][e % T];
}

// Thread 0 reads the status word; every thread gets the same answer.
__device__ bool block_failed(const int *status)
{
    __shared__ int f;
    __syncthreads();
    if (threadIdx.x == 0) f = ld_acquire(status) != 0;
    __syncthreads();
    return f != 0;
}

// After the CTA barrier, thread 0's release store orders every thread's
// earlier writes (the barrier puts them before it) ahead of the flag.
__device__ __forceinline__ void block_release(int *flag, int epoch)
{
    __syncthreads();
    if (threadIdx.x == 0) st_release(flag, epoch);
}

// Warp 4 of the panel during a factor (it shares warp 0's sub-partition, has
// no part in the plan and skips the factor's phase barriers): it raises the
// flags of the previous step's outputs (stored before that step ended; the
// release store waits for them here, off the pivot chain), then waits for
// the flags of the next step's tiles (the sub-diagonal SUB(I) and the
// diagonal PD(I+1) with its b) and copies those tiles into staging buffers.
// It stops waiting when the factor is done (*fdone, set by thread 0 after
// the last phase) or its budget runs out; *done says whether the tiles are
// there, else the panel loads them itself after the factor.
struct PanelSide {
    int *rel0, *rel1;          // flags to raise (null: none)
    const int *fa, *fb;        // flags the next tiles need (null: none)
    const double *Smat, *rhs;
    double (*asub)[T + 1], (*anext)[T + 1];
    double *bnext;
    int *done;
    int epoch, Np, I;
    bool want;                 // a next step exists

    __device__ void run(const int *fdone)
    {
        const int lane = threadIdx.x & 31;
        if (lane == 0) {
            if (rel0) st_release(rel0, epoch);
            if (rel1) st_release(rel1, epoch);
        }
        if (!want) return;
        bool up = false;
        const long long limit = s_spin_limit;
        for (long long it = 0; it < limit; ++it) {
            // every lane acquires the flags itself, so its own loads below are ordered after them
            up = (fa == nullptr || ld_acquire(fa) == epoch) && (fb == nullptr || ld_acquire(fb) == epoch);
            if (up || *(const volatile int *)fdone) break;
            __nanosleep(64);
        }
        if (!up) return;
        for (int e = lane; e < 2 * TT; e += 32) {
            const int t = e / TT, r = (e % TT) / T, c = e % T;
            const double v = __ldcg(Smat + (size_t)((I + 1) * T + r) * Np + (I + t) * T + c);
            if (t == 0) asub[r][c] = v;
            else anext[r][c] = v;
        }
        if (lane < T) bnext[lane] = __ldcg(rhs + (I + 1) * T + lane);
        __syncwarp();
        if (lane == 0) *done = 1;
    }
};

// Flags: tile (I, K) at tile_task(I, K); that slot is raised for the
// diagonal tile (I, I) when L_II, its inverse and y_I are stored, and for the
// sub-diagonal tile (I+1, I) when L_{I+1,I} is stored.  The partial diagonal
// PD(I) = A_II - sum_{J <= I-2} L_IJ L_IJ^T (with b_I likewise) raises
// n_fact + I; the partial sub-diagonal SUB(I) = A_{I+1,I} - sum_{J <= I-1}
// L_{I+1,J} L_IJ^T raises n_fact + nb + I; the second-subdiagonal tile
// (K+2, K) raises n_fact + 2 nb + K when its accumulation (before its solve)
// is in pre[K].
//
// The factor with the forward solve of rhs carried along.  CTA 0 (the panel)
// walks the diagonal: step I applies the last update to PD(I) with L_{I,I-1}
// (its own, kept in shared memory), factors the tile (cta_potrf), forms
// L_{I+1,I} = SUB(I) Linv_II^T and keeps it, then stores L_II, Linv_II, y_I
// and L_{I+1,I}.  The other CTAs (helpers) run the task list: the tiles
// (I, K) with I >= K + 2 (left-looking updates, then the triangular solve
// with Linv_KK), and the PD and SUB accumulations, in the order
//   P(0), C(0), PD(2), SUB(1), P(1), C(1), PD(3), SUB(2), P(2), ...
// (P = panel step, C(K) = the tiles of column K) -- every task depends only on
// tasks before it, each helper takes every (G-1)-th task in that order and
// the panel its steps in order, so with all CTAs resident (cooperative
// launch) the first unfinished task can always run: no deadlock.
__global__ void __launch_bounds__(CF_THREADS, 1) k_chol_dataflow(int Np, int nb, int n_tasks,
                                                              const int2 *__restrict__ tasks,
                                                              double *__restrict__ S,
                                                              double *__restrict__ Linv,
                                                              double *__restrict__ rhs,
                                                              double *__restrict__ pre,
                                                              int *__restrict__ flags, int epoch,
                                                              int *__restrict__ status, long long spin_limit)
{
    static_assert(BJ >= 6, "the panel keeps six tiles in the staging area");
    static_assert(LowerUpdate<true>::PART <= BJ * T * (T + 1), "update_lower's partial sums fit in the staging area");
    __shared__ double a[T][T + 1], linv[T][T + 1];
    __shared__ double bi[BJ][T][T + 1], bk[BJ][T][T + 1], by[BJ][T];
    __shared__ double bvec[T];
    __shared__ int ready_n;
    const int n_fact = nb * (nb + 1) / 2;
    const int tid = threadIdx.x;
    double *part = &bk[0][0][0];
    if (tid == 0) s_spin_limit = spin_limit;
    __syncthreads();
    if (blockIdx.x == 0) {
        // ---- panel.  Step I: warp 4 stores step I-1's outputs (L_{I-1,I-1},
        // its inverse, y_{I-1}, L_{I,I-1}) and raises their flags while the
        // other warps apply the last update to the diagonal tile; during the
        // factor warp 4 fetches the tiles of step I+1 (PanelSide); then
        // L_{I+1,I} is formed.  The panel tracks failure itself (a bad pivot of
        // its own, a wait that ran out), so it never reads the status word.
        double(*lsub)[T + 1] = bi[2];  // L_{I,I-1} from the previous step
        double(*asub)[T + 1] = bi[3];
        static_assert(LowerUpdate<true>::PART <= 2 * T * (T + 1) && LowerUpdate<true, CF_THREADS - 32>::PART <= 2 * T * (T + 1),
                      "update_lower's partial sums fit in bk[0..1]");
        static_assert(2 * T * (T + 1) + PW_SIZE <= BJ * T * (T + 1), "the factor workspace fits after the partial sums");
        double *W = &bk[2][0][0];  // bk[0..1] hold update_lower's partial sums
        double(*wa)[T + 1] = reinterpret_cast<double(*)[T + 1]>(W + PW_A);
        double(*wl)[T + 1] = reinterpret_cast<double(*)[T + 1]>(W + PW_L);
        double(*wli)[T + 1] = reinterpret_cast<double(*)[T + 1]>(W + PW_LINV);
        double(*anext)[T + 1] = bi[5];  // the next diagonal tile, fetched during the factor
        double *bnext = by[0];
        __shared__ PfPlan s_pf;
        __shared__ int pf_done;
        load_pf_plan(s_pf);
        bool failed = false;
        const int warp = tid >> 5, lane = tid & 31;
        load_tile(wa, S, Np, 0, 0);
        if (tid < T) W[PW_B + tid] = __ldcg(rhs + tid);
        __syncthreads();
        for (int I = 0; I < nb; ++I) {
            const int td = tile_task(I, I, nb);
            if (I >= 1) {
                // warp 4 stores step I-1's outputs and raises their flags (its
                // release waits for the stores, off the pivot chain) while the
                // other warps apply the last update to the diagonal tile
                if (warp == 4) {
                    if (!failed) {
                        const int Jp = I - 1;
                        for (int e2 = lane; e2 < TT; e2 += 32) {
                            const int r = e2 / T, c = e2 % T;
                            S[(size_t)(Jp * T + r) * Np + Jp * T + c] = wl[r][c];
                            Linv[(size_t)Jp * TT + e2] = wli[r][c];
                            S[(size_t)(I * T + r) * Np + Jp * T + c] = lsub[r][c];
                        }
                        if (lane < T) rhs[Jp * T + lane] = W[PW_Y + lane];
                    }
                    __syncwarp();
                    if (lane == 0) {
                        st_release(flags + tile_task(I - 1, I - 1, nb), epoch);
                        st_release(flags + tile_task(I, I - 1, nb), epoch);
                    }
                } else if (!failed) {
                    update_lower_panel(wa, lsub, W + PW_B, W + PW_Y);
                }
            }
            if (tid == 0) pf_done = 0;
            if (!failed) {
                PanelSide side{nullptr, nullptr,
                               I >= 1 ? flags + n_fact + nb + I : nullptr,
                               I + 1 >= 2 ? flags + n_fact + I + 1 : nullptr,
                               S, rhs, asub, anext, bnext, &pf_done, epoch, Np, I, I + 1 < nb};
                const bool good = cta_potrf(W, s_pf, side);
                if (!good) {
                    failed = true;
                    if (tid == 0) atomicCAS(status, 0, 1);
                }
            } else {
                __syncthreads();
            }
            if (I + 1 < nb) {
                // the tile and b are free after the factor: the next diagonal tile goes there
                if (pf_done) {
                    for (int e2 = tid; e2 < TT; e2 += CF_THREADS) wa[e2 / T][e2 % T] = anext[e2 / T][e2 % T];
                    if (tid < T) W[PW_B + tid] = bnext[tid];
                } else {
                    if (I >= 1 && !block_wait(flags + n_fact + nb + I, epoch, status)) failed = true;
                    if (I + 1 >= 2 && !block_wait(flags + n_fact + I + 1, epoch, status)) failed = true;
                    for (int e2 = tid; e2 < TT; e2 += CF_THREADS) {
                        const int r = e2 / T, c = e2 % T;
                        asub[r][c] = __ldcg(S + (size_t)((I + 1) * T + r) * Np + I * T + c);
                        wa[r][c] = __ldcg(S + (size_t)((I + 1) * T + r) * Np + (I + 1) * T + c);
                    }
                    if (tid < T) W[PW_B + tid] = __ldcg(rhs + (I + 1) * T + tid);
                }
                __syncthreads();
                if (!failed) tile_trsm(lsub, asub, wli);
                __syncthreads();
            }
        }
        // the last step's outputs
        if (!failed) {
            store_tile(S, Np, nb - 1, nb - 1, wl);
            for (int e2 = tid; e2 < TT; e2 += CF_THREADS) Linv[(size_t)(nb - 1) * TT + e2] = wli[e2 / T][e2 % T];
            if (tid < T) rhs[(nb - 1) * T + tid] = W[PW_Y + tid];
        }
        __syncthreads();
        if (tid == 0) st_release(flags + tile_task(nb - 1, nb - 1, nb), epoch);
        return;
    }
    // ---- helpers
    for (int t = blockIdx.x - 1; t < n_tasks; t += gridDim.x - 1) {
        const int I = tasks[t].x, K = tasks[t].y;
        const int kind = I - K;  // 0: PD(I), 1: SUB(K), >= 2: tile (I, K)
        const int mark = kind == 0 ? n_fact + I : kind == 1 ? n_fact + nb + K : tile_task(I, K, nb);
        load_tile(a, S, Np, I, K);
        if (kind == 0 && tid < T) bvec[tid] = __ldcg(rhs + I * T + tid);
        __syncthreads();
        // Updates J = 0 .. n_upd-1 in order.  The flags of the next BJ steps
        // are polled at once (one L2 round trip); the ready ones have all their
        // tiles loaded together and are applied from shared memory.  Each
        // element is updated in the same order as one step at a time would.
        const int n_upd = kind == 0 ? I - 1 : K;
        const int n_main = kind <= 1 ? n_upd - 1 : n_upd;  // PD and SUB take their last step below
        int J = 0;
        while (J < n_main) {
            const int nmax = min(BJ, n_main - J);
            if (tid == 0) ready_n = nmax;
            __syncthreads();
            if (tid < nmax) {
                const bool ok = ld_acquire(flags + tile_task(I, J + tid, nb)) == epoch &&
                                (kind == 0 || ld_acquire(flags + tile_task(K, J + tid, nb)) == epoch);
                if (!ok) atomicMin(&ready_n, tid);
            }
            __syncthreads();
            int n = ready_n;
            if (n == 0) {  // the next step is not done yet: wait for it alone
                block_wait(flags + tile_task(I, J, nb), epoch, status);
                if (kind != 0) block_wait(flags + tile_task(K, J, nb), epoch, status);
                n = 1;
            }
            for (int e2 = tid; e2 < n * TT; e2 += CF_THREADS) {
                const int q = e2 / TT, r = (e2 % TT) / T, c = e2 % T;
                bi[q][r][c] = __ldcg(S + (size_t)(I * T + r) * Np + (J + q) * T + c);
                if (kind != 0) bk[q][r][c] = __ldcg(S + (size_t)(K * T + r) * Np + (J + q) * T + c);
            }
            if (kind == 0)
                for (int e2 = tid; e2 < n * T; e2 += CF_THREADS) by[e2 / T][e2 % T] = __ldcg(rhs + (J + e2 / T) * T + e2 % T);
            __syncthreads();
            if (kind == 0) {
                // the partial sums use bk, which the diagonal accumulation leaves free
                for (int q = 0; q < n; ++q) update_lower<true>(a, bi[q], bvec, by[q], part);
            } else {
                for (int q = 0; q < n; ++q)
                    for (int e2 = tid; e2 < TT; e2 += CF_THREADS) {
                        const int r = e2 / T, c = e2 % T;
                        double sacc = a[r][c];
#pragma unroll
                        for (int k = 0; k < T; ++k) sacc = fma(-bi[q][r][k], bk[q][c][k], sacc);
                        a[r][c] = sacc;
                    }
            }
            __syncthreads();
            J += n;
        }
        if (kind <= 1) {
            // Last step, J = I - 2: L_{I,J} is the second-subdiagonal tile, whose
            // own task publishes it before its solve (PRE) and solves it once
            // the panel raises Linv_JJ.  PD and SUB solve it here themselves
            // (the same arithmetic, so the same bits) as soon as Linv_JJ is
            // up, which saves the panel a hand-off per step.
            const int Jl = I - 2;
            block_wait(flags + n_fact + 2 * nb + Jl, epoch, status);
            block_wait(flags + tile_task(Jl, Jl, nb), epoch, status);
            if (kind == 1) block_wait(flags + tile_task(K, Jl, nb), epoch, status);
            for (int e2 = tid; e2 < TT; e2 += CF_THREADS) {
                const int r = e2 / T, c = e2 % T;
                bi[1][r][c] = __ldcg(pre + (size_t)Jl * TT + e2);
                linv[r][c] = __ldcg(Linv + (size_t)Jl * TT + e2);
                if (kind == 1) bi[2][r][c] = __ldcg(S + (size_t)(K * T + r) * Np + Jl * T + c);
            }
            if (kind == 0 && tid < T) by[0][tid] = __ldcg(rhs + Jl * T + tid);
            __syncthreads();
            tile_trsm(bi[0], bi[1], linv);
            __syncthreads();
            if (kind == 0) {
                update_lower<true>(a, bi[0], bvec, by[0], part);
            } else {
                for (int e2 = tid; e2 < TT; e2 += CF_THREADS) {
                    const int r = e2 / T, c = e2 % T;
                    double sacc = a[r][c];
#pragma unroll
                    for (int k = 0; k < T; ++k) sacc = fma(-bi[0][r][k], bi[2][c][k], sacc);
                    a[r][c] = sacc;
                }
                __syncthreads();
            }
        } else if (kind == 2) {
            // the second-subdiagonal tile before its solve, for PD(K + 2) and SUB(K + 1)
            for (int e2 = tid; e2 < TT; e2 += CF_THREADS) pre[(size_t)K * TT + e2] = a[e2 / T][e2 % T];
            block_release(flags + n_fact + 2 * nb + K, epoch);
        }
        const bool failed = block_failed(status);
        if (kind == 0) {
            if (!failed) {
                store_tile(S, Np, I, I, a);
                if (tid < T) rhs[I * T + tid] = bvec[tid];
            }
        } else if (kind == 1) {
            if (!failed) store_tile(S, Np, I, K, a);
        } else {
            block_wait(flags + tile_task(K, K, nb), epoch, status);
            for (int e2 = tid; e2 < TT; e2 += CF_THREADS) linv[e2 / T][e2 % T] = __ldcg(Linv + (size_t)K * TT + e2);
            __syncthreads();
            if (!block_failed(status)) {
                tile_trsm(bi[0], a, linv);
                __syncthreads();
                store_tile(S, Np, I, K, bi[0]);
            }
        }
        block_release(flags + mark, epoch);
        __syncthreads();
    }
}

// Helper tasks in dependency order (see k_chol_dataflow): after panel step K
// come the tiles (I, K), I >= K + 2, then PD(K + 2) and SUB(K + 1).
void chol_task_list(int nb, std::vector<int2> &tasks)
{
    tasks.clear();
    for (int K = 0; K < nb; ++K) {
        for (int I = K + 2; I < nb; ++I) tasks.push_back(make_int2(I, K));
        if (K + 2 < nb) {
            tasks.push_back(make_int2(K + 2, K + 2));  // PD(K + 2)
            tasks.push_back(make_int2(K + 2, K + 1));  // SUB(K + 1)
        }
    }
}

int chol_grid(int n_tasks, int grid_cap)
{
    // CTAs per SM and SMs, per device (handles on several devices and
    // several host threads share this cache)
    static std::mutex mu;
    static int per_sm_dev[MAX_DEVICES], sms_dev[MAX_DEVICES];
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= MAX_DEVICES) dev = 0;
    int per_sm, sms;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (sms_dev[dev] == 0) {
            int p = 0, n = 0;
            cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&p, k_chol_dataflow, CF_THREADS, 0);
            if (p < 1) p = 1;
            if (PSBA_CHOL_PER_SM > 0 && p > PSBA_CHOL_PER_SM) p = PSBA_CHOL_PER_SM;
            per_sm_dev[dev] = p;
            sms_dev[dev] = n > 0 ? n : 1;
        }
        per_sm = per_sm_dev[dev];
        sms = sms_dev[dev];
    }
    int cap = per_sm * sms;
    if (grid_cap > 0 && grid_cap < cap) cap = grid_cap;
    if (cap < 2) cap = 2;  // the panel and at least one helper
    return n_tasks < cap ? n_tasks : cap;
}

// The back solve L^T x = rhs in one CTA of TS_THREADS threads with the
// right-hand side in shared memory (the factor's diagonal tasks already
// applied L^-1 to rhs); refine = 1: both solves of rhs, added into x.  A
// failed factor (status != 0) leaves x untouched.
constexpr int TS_THREADS = 512;

__global__ void __launch_bounds__(TS_THREADS) k_tri_solve(int refine, int Np, int nb, const double *__restrict__ S,
                                                           const double *__restrict__ Linv,
                                                           const double *__restrict__ rhs, double *__restrict__ x,
                                                           float2 *__restrict__ x2, const int *__restrict__ status)
{
    extern __shared__ double vec[];  // Np
    __shared__ double tmp[T];
    if (*status != 0) return;
    for (int i = threadIdx.x; i < Np; i += blockDim.x) vec[i] = rhs[i];
    __syncthreads();
    if (refine) cta_forward(Np, nb, S, Linv, vec, tmp);
    cta_back(Np, nb, S, Linv, vec, tmp, x, refine != 0, x2);
}

// ---------------------------------------------------------------------------
// The triangular solves on a thread-block cluster of TC_CTAS CTAs (one SM
// each): the back solve after the factor, or (refine = 1) both solves of a
// refinement residual, added into x.  One SM's FP64 rate bounds a one-CTA solve (N^2 / 2 multiply-adds);
// the cluster spreads the updates over TC_CTAS SMs and passes each step's
// solved block through distributed shared memory with one cluster barrier
// per step (~400 cycles on GB300, against 1-2 us for a flag in L2).
// Block I of the vector is owned by CTA I mod TC_CTAS, which holds it in
// shared memory.  Step K: the owner solves block K (16 x 16 product with
// the diagonal inverse, 256 threads, fixed shuffle tree), publishes it and
// arrives at the barrier; while the barrier completes, every CTA applies the
// previous step's block to its other blocks; after it, every CTA reads block
// K from the owner and first updates the block the next step needs (if it
// owns it), so the next owner can solve and arrive at once.  The diagonal
// inverse entries and the coefficients of both updates are loaded a step
// ahead, after the arrive.  The forward solve runs the same steps in the
// other direction over the rows of L.  Each vector entry takes its updates
// in step order: results do not depend on timing.
constexpr int TC_CTAS = 8, TC_THREADS = 256;

__device__ __forceinline__ void cl_arrive() { asm volatile("barrier.cluster.arrive.release.aligned;" ::: "memory"); }
__device__ __forceinline__ void cl_wait() { asm volatile("barrier.cluster.wait.acquire.aligned;" ::: "memory"); }

// v[c] -= sum_r P(r, c) xs[r] for the columns (back) or rows (forward) listed
// by idx(q), q < n: four threads per entry, four terms each, fixed tree.  The
// first pass (q < TC_THREADS / 4) takes its four coefficients from first[],
// loaded by the caller a step ahead; later passes load them here.
template <typename Coef, typename Idx>
__device__ __forceinline__ void cl_update(double *v, const double *xs, int n, const double (&first)[4], Coef coef,
                                          Idx idx)
{
    const int g = threadIdx.x & 3;
    for (int q0 = 0; q0 < n; q0 += TC_THREADS / 4) {
        const int q = q0 + (threadIdx.x >> 2);
        double s = 0.0;
        int c = 0;
        if (q < n) {
            c = idx(q);
            if (q0 == 0) {
#pragma unroll
                for (int j = 0; j < 4; ++j) s = fma(first[j], xs[4 * g + j], s);
            } else {
#pragma unroll
                for (int j = 0; j < 4; ++j) s = fma(coef(4 * g + j, c), xs[4 * g + j], s);
            }
        }
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (q < n && g == 0) v[c] -= s;
    }
}

__global__ void __launch_bounds__(TC_THREADS) k_tri_cluster(int refine, int Np, int nb,
                                                            const double *__restrict__ S,
                                                            const double *__restrict__ Linv,
                                                            const double *__restrict__ rhs,
                                                            double *__restrict__ x, float2 *__restrict__ x2,
                                                            const int *__restrict__ status)
{
    static_assert(TC_THREADS == TT, "one thread per term of the 16 x 16 diagonal product");
    extern __shared__ double vec[];  // Np; this CTA's blocks are the valid ones
    __shared__ double xb[2][T], xs[2][T];
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank(), tid = threadIdx.x;
    if (*status != 0) return;  // the same word for every CTA: all leave together
    for (int I = rank; I < nb; I += TC_CTAS)
        if (tid < T) vec[I * T + tid] = rhs[I * T + tid];
    const int dr = tid / T, dk = tid % T;
    const int cq = tid >> 2, cg4 = tid & 3;  // one entry of a block, four terms (threads 0..63)
    auto mine = [&](int I) { return I >= 0 && I < nb && I % TC_CTAS == rank; };
    // my first block above lo, and the entries of my blocks I with lo < I < hi
    auto first_above = [&](int lo) { return lo < rank ? rank : rank + ((lo - rank) / TC_CTAS + 1) * TC_CTAS; };
    auto n_between = [&](int lo, int hi) {
        const int f = first_above(lo);
        return f < hi ? ((hi - 1 - f) / TC_CTAS + 1) * T : 0;
    };
    auto entry_between = [&](int lo, int q) {  // q-th entry of my blocks above lo, ascending
        return (first_above(lo) + (q / T) * TC_CTAS) * T + q % T;
    };
    // the next step's block update, from coefficients loaded a step ahead
    auto crit_apply = [&](const double *xs_, const double (&cf)[4], int entry) {
        double s = 0.0;
#pragma unroll
        for (int j = 0; j < 4; ++j) s = fma(cf[j], xs_[4 * cg4 + j], s);
        s += __shfl_xor_sync(0xffffffffu, s, 1);
        s += __shfl_xor_sync(0xffffffffu, s, 2);
        if (cq < T && cg4 == 0) vec[entry] -= s;
    };
    __syncthreads();
    // Every register loaded for the next step goes to the other half of a
    // ping-pong pair (the loop is unrolled by two), so nothing waits for a
    // load until the step that uses it; all loads are issued after the
    // arrive (a load in flight at the arrive would hold up its release).
    if (refine) {
        // L y = b: step K solves y_K = Linv_K b_K, then b_I -= L_IK y_K for I > K
        auto ldiag = [&](int K) {
            return mine(K) && dk <= dr ? __ldcg(Linv + (size_t)K * TT + dr * T + dk) : 0.0;
        };
        auto lcrit = [&](int K, double (&cf)[4]) {  // rows of block K+1, columns of block K
#pragma unroll
            for (int j = 0; j < 4; ++j)
                cf[j] = (cq < T && mine(K + 1)) ? __ldcg(S + (size_t)((K + 1) * T + cq) * Np + K * T + 4 * cg4 + j)
                                                : 0.0;
        };
        auto ldef = [&](int P, double (&df)[4]) {  // rows of my blocks above P + 1, columns of block P
            const int n = n_between(P + 1, nb);
            const int i = cq < n ? entry_between(P + 1, cq) : 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) df[j] = cq < n ? __ldcg(S + (size_t)i * Np + P * T + 4 * cg4 + j) : 0.0;
        };
        int pend = -1;
        auto step = [&](int K, double &pl, double &pln, double (&cf)[4], double (&cfn)[4], double (&df)[4],
                        double (&dfn)[4]) {
            if (mine(K)) {
                const double yv = half_warp_sum(pl * vec[K * T + dk]);
                if (dk == 0) xb[K & 1][dr] = yv;
            }
            __syncthreads();
            if (mine(K) && tid < T) vec[K * T + tid] = xb[K & 1][tid];
            cl_arrive();
            pln = K + 1 < nb ? ldiag(K + 1) : 0.0;
            lcrit(K + 1, cfn);
            ldef(K, dfn);
            if (pend >= 0) {  // the previous step's block, applied to my blocks above pend + 1
                const int P = pend;
                cl_update(vec, xs[P & 1], n_between(P + 1, nb), df,
                          [&](int r, int i) { return __ldcg(S + (size_t)i * Np + P * T + r); },
                          [&](int q) { return entry_between(P + 1, q); });
            }
            cl_wait();
            if (tid < T) xs[K & 1][tid] = cl.map_shared_rank(&xb[K & 1][0], K % TC_CTAS)[tid];
            __syncthreads();
            if (mine(K + 1)) crit_apply(xs[K & 1], cf, (K + 1) * T + cq);
            __syncthreads();
            pend = K;
        };
        double plA = ldiag(0), plB = 0.0, cfA[4], cfB[4], dfA[4] = {0.0, 0.0, 0.0, 0.0}, dfB[4];
        lcrit(0, cfA);
        for (int K = 0; K < nb; K += 2) {
            step(K, plA, plB, cfA, cfB, dfA, dfB);
            if (K + 1 < nb) step(K + 1, plB, plA, cfB, cfA, dfB, dfA);
        }
        // the last step's block reaches no block above it; every CTA has read
        // it before the back solve's first step rewrites its buffer
        cl_arrive();
        cl_wait();
    }
    {
        // L^T x = y: step K solves x_K = Linv_K^T y_K, then y_I -= L_KI^T x_K for I < K
        auto ldiag = [&](int K) {
            return mine(K) && dk >= dr ? __ldcg(Linv + (size_t)K * TT + dk * T + dr) : 0.0;
        };
        auto lcrit = [&](int K, double (&cf)[4]) {  // rows of block K, columns of block K-1
#pragma unroll
            for (int j = 0; j < 4; ++j)
                cf[j] = (cq < T && mine(K - 1)) ? __ldcg(S + (size_t)(K * T + 4 * cg4 + j) * Np + (K - 1) * T + cq)
                                                : 0.0;
        };
        auto ldef = [&](int P, double (&df)[4]) {  // rows of block P, columns of my blocks below P - 1
            const int n = n_between(-1, P - 1);
            const int c = cq < n ? entry_between(-1, cq) : 0;
#pragma unroll
            for (int j = 0; j < 4; ++j) df[j] = cq < n ? __ldcg(S + (size_t)(P * T + 4 * cg4 + j) * Np + c) : 0.0;
        };
        int pend = -1;
        auto step = [&](int K, double &pl, double &pln, double (&cf)[4], double (&cfn)[4], double (&df)[4],
                        double (&dfn)[4]) {
            if (mine(K)) {
                const double xv = half_warp_sum(pl * vec[K * T + dk]);
                if (dk == 0) xb[K & 1][dr] = xv;
            }
            __syncthreads();
            // x_K replaces y_K in the owner's vector (no global store before the release)
            if (mine(K) && tid < T) vec[K * T + tid] = xb[K & 1][tid];
            cl_arrive();
            pln = K > 0 ? ldiag(K - 1) : 0.0;
            lcrit(K - 1, cfn);
            ldef(K, dfn);
            if (pend >= 0) {  // the previous step's block, applied to my blocks below pend - 1
                const int P = pend;
                cl_update(vec, xs[P & 1], n_between(-1, P - 1), df,
                          [&](int r, int c) { return __ldcg(S + (size_t)(P * T + r) * Np + c); },
                          [&](int q) { return entry_between(-1, q); });
            }
            cl_wait();
            if (tid < T) xs[K & 1][tid] = cl.map_shared_rank(&xb[K & 1][0], K % TC_CTAS)[tid];
            __syncthreads();
            if (mine(K - 1)) crit_apply(xs[K & 1], cf, (K - 1) * T + cq);
            __syncthreads();
            pend = K;
        };
        double plA = ldiag(nb - 1), plB = 0.0, cfA[4], cfB[4], dfA[4] = {0.0, 0.0, 0.0, 0.0}, dfB[4];
        lcrit(nb - 1, cfA);
        for (int K = nb - 1; K >= 0; K -= 2) {
            step(K, plA, plB, cfA, cfB, dfA, dfB);
            if (K - 1 >= 0) step(K - 1, plB, plA, cfB, cfA, dfB, dfA);
        }
        // no CTA may leave while another can still read its shared memory
        cl_arrive();
        cl_wait();
        for (int I = rank; I < nb; I += TC_CTAS)
            if (tid < T) {
                const double xv = refine ? x[I * T + tid] + vec[I * T + tid] : vec[I * T + tid];
                x[I * T + tid] = xv;
                if (x2) x2[I * T + tid] = split2f(xv);
            }
    }
}

// The triangular solves after the factor: the back solve of d.rhs into x
// (refine = 0), or both solves of d.rhs added into x (refine = 1).
void launch_tri(const DeviceProblem &d, int refine, double *x, cudaStream_t s)
{
    const int nb = d.Np / T, Np = d.Np;
    // the solution also as FP32 pairs for the mixed form's eb sums (x is dpa
    // on every path that reaches them)
    float2 *x2 = d.prec == PSBA_PREC_MIXED && d.cnp == 6 ? d.dpa2f : nullptr;
#if PSBA_TRI_CLUSTER
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(TC_CTAS);
    cfg.blockDim = dim3(TC_THREADS);
    cfg.dynamicSmemBytes = sizeof(double) * Np;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = TC_CTAS;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    const double *S = d.S, *Linv = d.Linv, *rhs = d.rhs;
    cudaLaunchKernelEx(&cfg, k_tri_cluster, refine, Np, nb, S, Linv, rhs, x, x2, (const int *)d.status);
#else
    k_tri_solve<<<1, TS_THREADS, sizeof(double) * Np, s>>>(refine, Np, nb, d.S, d.Linv, d.rhs, x, x2, d.status);
#endif
    note_launch(1);
}

void launch_chol_dataflow(const DeviceProblem &d, int epoch, double *x_out, cudaStream_t s)
{
    int nb = d.Np / T;
    int Np = d.Np;
    {
        int n_tasks = d.chol_n_tasks;
        const int grid = chol_grid(n_tasks + 1, d.chol_grid_cap);
        const int2 *tasks = d.chol_tasks;
        double *S = d.S, *Linv = d.Linv, *rhs = d.rhs, *pre = d.chol_pre;
        int *flags = d.chol_flags, *status = d.status;
        long long spin = d.wait_limit;
        void *args[] = {&Np, &nb, &n_tasks, (void *)&tasks, &S, &Linv, &rhs, &pre, &flags, &epoch, &status, &spin};
        cudaMemsetAsync(d.status, 0, 2 * sizeof(int), s);
        cudaLaunchCooperativeKernel((const void *)k_chol_dataflow, dim3(grid), dim3(CF_THREADS), args, 0, s);
        note_launch(1);
    }
    launch_tri(d, 0, x_out, s);
}

// r = b - S x over the Np rows (S symmetric, its lower triangle in Sc with
// leading dimension ld), each row's sum as Dot2 of Ogita, Rump and Oishi
// ("Accurate sum and dot product", SIAM J. Sci. Comput. 26(6), 2005): every
// product split exactly by an FMA, the running sum carried with Knuth's
// TwoSum and the rounding errors summed beside it, so the residual is as
// accurate as if S x were formed in twice the working precision.  A residual
// formed in plain FP64 is mostly the rounding of S x (S x matches b to the
// last bits after a backward-stable solve), so a refinement step on it
// leaves the forward error where it was; on this one it falls from ~cond(S)
// eps to ~eps.  One warp a row: the row's part left of the diagonal and the
// column's part below it, each lane's terms in order, then a fixed xor tree
// of the (sum, error) pairs.  A failed factor (status != 0) leaves r
// untouched.
constexpr int RR_THREADS = 256;

// s + e = a + b exactly (Knuth's TwoSum)
__device__ __forceinline__ void two_sum(double a, double b, double &s, double &e)
{
    s = __dadd_rn(a, b);
    const double z = __dsub_rn(s, a);
    e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, z)), __dsub_rn(b, z));
}

// (hi, lo) += a x
__device__ __forceinline__ void dot2_add(double a, double x, double &hi, double &lo)
{
    const double p = __dmul_rn(a, x);
    const double pe = fma(a, x, -p);  // a x - p exactly
    double t;
    two_sum(hi, p, hi, t);
    lo = __dadd_rn(lo, __dadd_rn(t, pe));
}

__global__ void __launch_bounds__(RR_THREADS) k_refine_residual(int Np, const double *__restrict__ Sc, int ld,
                                                                 const double *__restrict__ b,
                                                                 const double *__restrict__ x, double *__restrict__ r,
                                                                 const int *__restrict__ status)
{
    const int i = (int)((blockIdx.x * (size_t)RR_THREADS + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (i >= Np || *status != 0) return;
    const double *row = Sc + (size_t)i * ld;
    double hi = 0.0, lo = 0.0;
    for (int j = lane; j <= i; j += 32) dot2_add(row[j], x[j], hi, lo);
    for (int j = i + 1 + lane; j < Np; j += 32) dot2_add(Sc[(size_t)j * ld + i], x[j], hi, lo);
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        const double oh = __shfl_xor_sync(0xffffffffu, hi, off), ol = __shfl_xor_sync(0xffffffffu, lo, off);
        double t;
        two_sum(hi, oh, hi, t);
        lo = __dadd_rn(__dadd_rn(lo, ol), t);
    }
    if (lane == 0) {
        double s, t;
        two_sum(b[i], -hi, s, t);
        r[i] = __dadd_rn(s, __dsub_rn(t, lo));
    }
}

// One refinement step of the solve x of S x = b just made: S and b were saved
// (Sc with leading dimension ld, bc) before the factor overwrote them; the
// residual goes to d.rhs, and its solve is added into x.
void launch_refine(const DeviceProblem &d, const double *Sc, int ld, const double *bc, double *x, cudaStream_t s)
{
    const int blocks = (int)(((size_t)d.Np * 32 + RR_THREADS - 1) / RR_THREADS);
    k_refine_residual<<<blocks, RR_THREADS, 0, s>>>(d.Np, Sc, ld, bc, x, d.rhs, d.status);
    note_launch(1);
    launch_tri(d, 1, x, s);
}

// ---------------------------------------------------------------------------
// Modified Cholesky (trust-region lambda fallback), restating cholmod_blk.cl
// with get_delta_beta (cl_cholmod.cpp:109-165) and kern_cholmod_E: block
// columns of 3 are factored as plain 3x3 blocks when the pivots are positive
// and every entry below is <= beta; otherwise their columns are redone one
// at a time with d = max(|c|, delta) and the theta/beta bound.
//
// One cooperative launch over CM_CTAS CTAs (grid-wide barriers), right-
// looking: step j factors the 3x3 diagonal block of the already updated
// matrix (every CTA redundantly, the same arithmetic), writes the panel
// below it (a 3x3 block per thread) and, after a grid barrier that also
// combines the "entry above beta" flags, updates the trailing lower triangle
// with the rank-3 product of the panel (rows dealt to CTAs, columns to
// threads).  Each entry thus takes the same sequence of 3-term subtractions,
// in the same block order, as the reference's left-looking sums, so the plain
// path rounds as before; the column-at-a-time path subtracts the earlier
// blocks in those 3-term groups and the block's own columns one at a time.
// The work per step is spread over the GPU instead of one block of threads
// (at N = 528: ~33 ms on one CTA, where a step had at most 175 threads busy).
constexpr int CM_THREADS = 256;

__device__ double cta_max(double v, double *red)
{
    for (int off = 16; off > 0; off >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    double r = red[0];
    for (int w = 1; w < CM_THREADS / 32; ++w) r = fmax(r, red[w]);
    __syncthreads();
    return r;
}

__device__ int cta_or(int v, int *red)
{
    v = __any_sync(0xffffffffu, v) ? 1 : 0;
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    int r = 0;
    for (int w = 0; w < CM_THREADS / 32; ++w) r |= red[w];
    __syncthreads();
    return r;
}

// work: diag (n), orig (3 n), C (n), then gmax[2 G] and gflag[G] (doubles)
__global__ void __launch_bounds__(CM_THREADS) k_cholmod(double *S, int n, int ld, double *E, double *work)
{
    cg::grid_group grid = cg::this_grid();
    __shared__ double dred[CM_THREADS / 32];
    __shared__ int ired[CM_THREADS / 32];
    __shared__ double sh_L[6], sh_Li[9], sh_lxx;
    __shared__ int sh_fail;
    const int G = gridDim.x, b = blockIdx.x, tid = threadIdx.x;
    const long long gtid = (long long)b * CM_THREADS + tid, gsize = (long long)G * CM_THREADS;
    double *diag = work, *orig = work + n, *C = work + 4 * n, *gmax = work + 5 * n, *gflag = gmax + 2 * G;
    // a grid-wide OR / max through per-CTA slots (after a grid barrier every
    // CTA reads them all, in the same order)
    auto grid_or = [&](int v) {
        v = cta_or(v, ired);
        if (tid == 0) gflag[b] = v ? 1.0 : 0.0;
        grid.sync();
        int r = 0;
        for (int q = 0; q < G; ++q) r |= gflag[q] != 0.0;
        grid.sync();  // the slots are reused
        return r;
    };
    auto grid_max = [&](double v, int slot) {
        v = cta_max(v, dred);
        if (tid == 0) gmax[2 * b + slot] = v;
        grid.sync();
        double r = 0.0;
        for (int q = 0; q < G; ++q) r = fmax(r, gmax[2 * q + slot]);
        return r;
    };
    // xi = max |offdiag|, gamma = max |diag| over the symmetric matrix (lower read)
    double xi = 0.0, gam = 0.0;
    for (long long e = gtid; e < (long long)n * n; e += gsize) {
        const int r = (int)(e / n), k = (int)(e % n);
        if (r == k) {
            gam = fmax(gam, fabs(S[(size_t)r * ld + r]));
        } else {
            const int hi = r > k ? r : k, lo = r > k ? k : r;
            xi = fmax(xi, fabs(S[(size_t)hi * ld + lo]));
        }
    }
    for (long long r = gtid; r < n; r += gsize) diag[r] = S[(size_t)r * ld + r];
    xi = cta_max(xi, dred);
    gam = cta_max(gam, dred);
    if (tid == 0) {
        gmax[2 * b] = xi;
        gmax[2 * b + 1] = gam;
    }
    grid.sync();
    xi = 0.0;
    gam = 0.0;
    for (int q = 0; q < G; ++q) {
        xi = fmax(xi, gmax[2 * q]);
        gam = fmax(gam, gmax[2 * q + 1]);
    }
    grid.sync();
    const double delta = 1e-15 * fmax(xi + gam, 1.0);
    double beta = fmax(gam, 1e-15);
    beta = fmax(beta, xi / sqrt((double)(n * n - 1)));
    beta = sqrt(beta);
    const int nb = n / 3;
    for (int j = 0; j < nb; ++j) {
        const int j3 = 3 * j;
        // the diagonal block, already updated by the earlier steps
        if (tid == 0) {
            double Tm[9];
            for (int q = 0; q < 9; ++q) {
                const int u = q / 3, v = q % 3;
                Tm[q] = v > u ? S[(size_t)(j3 + v) * ld + j3 + u] : S[(size_t)(j3 + u) * ld + j3 + v];
            }
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
        const int fail = sh_fail;  // the same in every CTA
        // keep the column block (rows j3 .. n-1) for the column-at-a-time path
        for (long long e = gtid; e < (long long)(n - j3) * 3; e += gsize) {
            const int r = j3 + (int)(e / 3), v = (int)(e % 3);
            orig[(size_t)r * 3 + v] = S[(size_t)r * ld + j3 + v];
        }
        grid.sync();
        int redo = fail;
        if (!fail) {
            // the diagonal block, then the blocks below: L_ij = T_ij Li^T
            if (gtid == 0) {
                double *dd = S + (size_t)j3 * ld + j3;
                dd[0] = sh_L[0]; dd[1] = 0; dd[2] = 0;
                dd[ld] = sh_L[1]; dd[ld + 1] = sh_L[2]; dd[ld + 2] = 0;
                dd[2 * ld] = sh_L[3]; dd[2 * ld + 1] = sh_L[4]; dd[2 * ld + 2] = sh_L[5];
            }
            int big = 0;
            for (long long blk = j + 1 + gtid; blk < nb; blk += gsize) {
                double Tij[9];
                for (int q = 0; q < 9; ++q) Tij[q] = S[(size_t)(3 * blk + q / 3) * ld + j3 + q % 3];
                for (int u = 0; u < 3; ++u)
                    for (int v = 0; v < 3; ++v) {
                        const double val = (Tij[u * 3] * sh_Li[v * 3] + Tij[u * 3 + 1] * sh_Li[v * 3 + 1] +
                                            Tij[u * 3 + 2] * sh_Li[v * 3 + 2]);
                        S[(size_t)(3 * blk + u) * ld + j3 + v] = val;
                        S[(size_t)(j3 + v) * ld + 3 * blk + u] = 0.0;
                        if (val > beta) big = 1;
                    }
            }
            redo = grid_or(big);
        }
        if (redo) {
            // restore the column block and redo its columns one at a time
            for (long long e = gtid; e < (long long)(n - j3) * 3; e += gsize) {
                const int r = j3 + (int)(e / 3), v = (int)(e % 3);
                S[(size_t)r * ld + j3 + v] = orig[(size_t)r * 3 + v];
            }
            grid.sync();
            for (int col = 0; col < 3; ++col) {
                const int x = j3 + col;
                if (tid == 0) {  // every CTA, the same arithmetic
                    double sum = S[(size_t)x * ld + x];
                    for (int k = j3; k < x; ++k) {
                        const double l = S[(size_t)x * ld + k];
                        sum -= l * l;
                    }
                    sum = fabs(sum);
                    sh_lxx = sqrt(fmax(sum, delta));
                }
                __syncthreads();
                const double lxx = sh_lxx;
                int big = 0;
                for (long long i = x + 1 + gtid; i < n; i += gsize) {
                    double c = S[(size_t)i * ld + x];
                    for (int k = j3; k < x; ++k) c = c - (S[(size_t)i * ld + k] * S[(size_t)x * ld + k]);
                    C[i] = c;
                    const double l = c / lxx;
                    S[(size_t)i * ld + x] = l;
                    S[(size_t)x * ld + i] = 0.0;
                    if (l > beta) big = 1;
                }
                big = grid_or(big);  // also orders the column's writes before the next column
                if (gtid == 0) S[(size_t)x * ld + x] = lxx;
                if (big) {
                    double th = 0.0;
                    for (long long i = x + 1 + gtid; i < n; i += gsize) th = fmax(th, fabs(C[i]));
                    th = grid_max(th, 0);
                    const double nl = th / beta;
                    if (gtid == 0) S[(size_t)x * ld + x] = nl;
                    for (long long i = x + 1 + gtid; i < n; i += gsize) S[(size_t)i * ld + x] = C[i] / nl;
                }
                grid.sync();
            }
        }
        // the trailing lower triangle: S_ic -= L_i,j3.. L_c,j3.. (rank 3),
        // rows i dealt to CTAs, columns c to threads
        const int t0 = j3 + 3;
        for (int i = t0 + b; i < n; i += G) {
            const double *Li_ = S + (size_t)i * ld + j3;
            const double a0 = Li_[0], a1 = Li_[1], a2 = Li_[2];
            for (int c = t0 + tid; c <= i; c += CM_THREADS) {
                const double *Lc = S + (size_t)c * ld + j3;
                S[(size_t)i * ld + c] -= (a0 * Lc[0] + a1 * Lc[1] + a2 * Lc[2]);
            }
        }
        grid.sync();
    }
    for (long long i = gtid; i < n; i += gsize) {
        double sum = 0.0;
        for (int k = 0; k <= i; ++k) sum += S[(size_t)i * ld + k] * S[(size_t)i * ld + k];
        E[i] = sum - diag[i];
    }
}

// doubles of work the modified Cholesky needs at size n
size_t cholmod_work(int n) { return 5 * (size_t)n + 3 * (size_t)CM_MAX_CTAS + 8; }

void launch_cholmod(double *S, int n, int ld, double *E, double *work, cudaStream_t s, int grid_cap)
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int G = sms < CM_MAX_CTAS ? sms : CM_MAX_CTAS;
    if (grid_cap > 0 && grid_cap < G) G = grid_cap;
    const int rows = (n + 7) / 8;  // no more CTAs than the trailing rows can use
    if (rows < G) G = rows;
    if (G < 1) G = 1;
    void *args[] = {&S, &n, &ld, &E, &work};
    cudaLaunchCooperativeKernel((const void *)k_cholmod, dim3(G), dim3(CM_THREADS), args, 0, s);
    note_launch(1);
}

}  // namespace psba

// ---------------------------------------------------------------------------
// Diagnostic entry points for the parity tests: the dense solve on a caller
// matrix, and the pivot chain's reciprocal.
namespace psba {

__global__ void k_pivot_reciprocal(int n, const double *__restrict__ x, double *__restrict__ y)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) y[i] = rcp_fast(x[i]);
}

}  // namespace psba

extern "C" int psba_eval_pivot_reciprocal(int n, const double *x, double *y)
{
    using namespace psba;
    if (n < 0 || (n > 0 && (!x || !y))) return set_error("psba_eval_pivot_reciprocal: bad arguments"), PSBA_ERR_ARG;
    if (n == 0) return PSBA_OK;
    double *dx = nullptr, *dy = nullptr;
    cudaError_t e = cudaMalloc(&dx, sizeof(double) * (size_t)n);
    if (e == cudaSuccess) e = cudaMalloc(&dy, sizeof(double) * (size_t)n);
    if (e == cudaSuccess) e = cudaMemcpy(dx, x, sizeof(double) * (size_t)n, cudaMemcpyHostToDevice);
    if (e == cudaSuccess) {
        k_pivot_reciprocal<<<(n + 255) / 256, 256>>>(n, dx, dy);
        note_launch(1);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpy(y, dy, sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost);
    cudaFree(dx);
    cudaFree(dy);
    if (e != cudaSuccess) return set_error(std::string("CUDA error: ") + cudaGetErrorString(e)), PSBA_ERR_CUDA;
    return PSBA_OK;
}

// The handle's dense solve (k_chol_dataflow + the back solve) on an n x n
// matrix given by the caller: S row-major, lower triangle read; padded to a
// multiple of TILE with an identity block.
extern "C" int psba_eval_dense_solve(int n, const double *S, const double *b, double *x, int *status)
{
    using namespace psba;
    if (n <= 0 || n > 4096 || !S || !b || !x || !status)
        return set_error("psba_eval_dense_solve: n must be in 1..4096 and every pointer set"), PSBA_ERR_ARG;
    DeviceProblem d;
    d.Np = ((n + TILE - 1) / TILE) * TILE;
    const int Np = d.Np, nb = Np / TILE;
    std::vector<int2> tasks;
    chol_task_list(nb, tasks);
    d.chol_n_tasks = (int)tasks.size();
    d.chol_n_flags = nb * (nb + 1) / 2 + 3 * nb;
    std::vector<double> hS((size_t)Np * Np, 0.0), hb(Np, 0.0);
    for (int r = 0; r < Np; ++r)
        for (int c = 0; c <= r; ++c) hS[(size_t)r * Np + c] = (r < n && c < n) ? S[(size_t)r * n + c] : (r == c ? 1.0 : 0.0);
    for (int r = 0; r < n; ++r) hb[r] = b[r];
    cudaStream_t st = nullptr;
    std::vector<void *> mem;
    cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    auto get = [&](auto **p, size_t count) {
        if (e != cudaSuccess) return;
        e = cudaMalloc((void **)p, sizeof(**p) * (count ? count : 1));
        if (e == cudaSuccess) mem.push_back((void *)*p);
    };
    get(&d.S, (size_t)Np * Np);
    get(&d.rhs, (size_t)Np);
    get(&d.xsol, (size_t)Np);
    get(&d.Linv, (size_t)Np * TILE);
    get(&d.chol_pre, (size_t)nb * TILE * TILE);
    get(&d.chol_tasks, tasks.size());
    get(&d.chol_flags, (size_t)d.chol_n_flags);
    get(&d.status, 4);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.S, hS.data(), sizeof(double) * hS.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(d.rhs, hb.data(), sizeof(double) * Np, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && !tasks.empty())
        e = cudaMemcpyAsync(d.chol_tasks, tasks.data(), sizeof(int2) * tasks.size(), cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.chol_flags, 0, sizeof(int) * d.chol_n_flags, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d.status, 0, sizeof(int) * 4, st);
    if (e == cudaSuccess) {
        launch_chol_dataflow(d, 1, d.xsol, st);
        e = cudaGetLastError();
    }
    int hst[4] = {0, 0, 0, 0};
    if (e == cudaSuccess) e = cudaMemcpyAsync(hst, d.status, sizeof(hst), cudaMemcpyDeviceToHost, st);
    std::vector<double> hx(Np);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hx.data(), d.xsol, sizeof(double) * Np, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    for (void *p : mem) cudaFree(p);
    if (st) cudaStreamDestroy(st);
    if (e != cudaSuccess) return set_error(std::string("CUDA error: ") + cudaGetErrorString(e)), PSBA_ERR_CUDA;
    *status = hst[0];
    if (hst[0] == 0)
        for (int r = 0; r < n; ++r) x[r] = hx[r];
    return PSBA_OK;
}

// Dense FP64 reduced-camera solve on sm_103a: blocked right-looking
// Cholesky of S (Np x Np, lower triangle, Np a multiple of TILE) with the
// forward solve L y = ea carried along as an extra column, then the back
// solve L^T x = y.
//
// This replaces the reference's explicit inverse (SPD_inv.cl: 3x3-block
// Cholesky, kern_trigMat_inv, kern_trigMat_mul, then matVec_mul) with two
// triangular solves: fewer flops and no N^2 inverse in memory.  The failure
// test is the reference's: a non-positive or non-finite pivot sets the status
// word (SPD_inv.cl:66-107) and every later kernel of the sweep returns early.
//
// Per step J: trsm(J) computes the panel L_IJ = A_IJ L_JJ^-T (one block per
// tile), update(J) applies A_IK -= L_IJ L_KJ^T to the trailing tiles and the
// block that owns tile (J+1, J+1) factors it right away.
#include "psba_internal.h"

namespace psba {

constexpr int T = TILE;
constexpr int TT = TILE * TILE;

// Factor the tile in shared memory a[T][T+1] (lower), compute its inverse
// linv and y = linv * b.  Returns false (and sets *status) on a bad pivot.
__device__ bool tile_potrf(double (*a)[T + 1], double (*linv)[T + 1], const double *b, double *y,
                           int *status)
{
    __shared__ int bad;
    const int tid = threadIdx.x;
    if (tid == 0) bad = 0;
    __syncthreads();
    for (int k = 0; k < T; ++k) {
        if (tid == 0) {
            const double d = a[k][k];
            if (!(d > 0.0) || !isfinite(d)) {
                bad = 1;
            } else {
                a[k][k] = sqrt(d);
            }
        }
        __syncthreads();
        if (bad) break;
        const double piv = a[k][k];
        for (int i = k + 1 + tid; i < T; i += blockDim.x) a[i][k] = a[i][k] / piv;
        __syncthreads();
        const int m = T - k - 1;  // trailing size
        for (int e = tid; e < m * m; e += blockDim.x) {
            const int i = k + 1 + e / m, j = k + 1 + e % m;
            if (j <= i) a[i][j] = a[i][j] - a[i][k] * a[j][k];
        }
        __syncthreads();
    }
    if (bad) {
        if (tid == 0) *status = 1;
        return false;
    }
    // inverse of the lower-triangular factor, one column per thread
    if (tid < T) {
        const int c = tid;
        for (int i = 0; i < c; ++i) linv[i][c] = 0.0;
        linv[c][c] = 1.0 / a[c][c];
        for (int i = c + 1; i < T; ++i) {
            double s = 0.0;
            for (int k = c; k < i; ++k) s = fma(a[i][k], linv[k][c], s);
            linv[i][c] = -s / a[i][i];
        }
    }
    __syncthreads();
    if (tid < T) {
        double s = 0.0;
        for (int k = 0; k <= tid; ++k) s = fma(linv[tid][k], b[k], s);
        y[tid] = s;
    }
    __syncthreads();
    return true;
}

// Store a factored diagonal tile, its inverse and y.
__device__ void tile_store_diag(double (*a)[T + 1], double (*linv)[T + 1], const double *y, int J,
                                int Np, double *S, double *Linv, double *rhs)
{
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int r = e / T, c = e % T;
        S[(size_t)(J * T + r) * Np + J * T + c] = c <= r ? a[r][c] : 0.0;
        Linv[(size_t)J * TT + e] = linv[r][c];
    }
    if (threadIdx.x < T) rhs[J * T + threadIdx.x] = y[threadIdx.x];
}

__global__ void __launch_bounds__(TT) k_chol_first(int Np, double *S, double *Linv, double *rhs,
                                                   int *status)
{
    __shared__ double a[T][T + 1], linv[T][T + 1], b[T], y[T];
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int r = e / T, c = e % T;
        a[r][c] = S[(size_t)r * Np + c];
    }
    if (threadIdx.x < T) b[threadIdx.x] = rhs[threadIdx.x];
    if (threadIdx.x == 0) *status = 0;
    __syncthreads();
    if (!tile_potrf(a, linv, b, y, status)) return;
    tile_store_diag(a, linv, y, 0, Np, S, Linv, rhs);
}

// L_IJ = A_IJ Linv_J^T for I = J+1 .. nb-1 (one block per tile).
__global__ void __launch_bounds__(TT) k_chol_trsm(int J, int Np, double *S, const double *Linv,
                                                  const int *status)
{
    if (*status) return;
    __shared__ double a[T][T + 1], li[T][T + 1];
    const int I = J + 1 + blockIdx.x;
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int r = e / T, c = e % T;
        a[r][c] = S[(size_t)(I * T + r) * Np + J * T + c];
        li[r][c] = Linv[(size_t)J * TT + e];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int r = e / T, c = e % T;
        double s = 0.0;
        for (int k = 0; k <= c; ++k) s = fma(a[r][k], li[c][k], s);
        S[(size_t)(I * T + r) * Np + J * T + c] = s;
    }
}

// Trailing update after step J: tiles (I, K), J < K <= I < nb, plus the
// right-hand side; the block of tile (J+1, J+1) then factors it.
__global__ void __launch_bounds__(TT) k_chol_update(int J, int nb, int Np, double *S, double *Linv,
                                                    double *rhs, int *status)
{
    if (*status) return;
    __shared__ double li[T][T + 1], lk[T][T + 1], a[T][T + 1], linv[T][T + 1], b[T], y[T];
    // tile index -> (I, K) over the lower triangle of the trailing matrix
    const int m = nb - J - 1;
    int t = blockIdx.x, I = 0, K = 0;
    {
        int row = 0;
        while (t >= row + 1) {
            t -= row + 1;
            ++row;
        }
        I = J + 1 + row;
        K = J + 1 + t;
    }
    (void)m;
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int r = e / T, c = e % T;
        li[r][c] = S[(size_t)(I * T + r) * Np + J * T + c];
        lk[r][c] = S[(size_t)(K * T + r) * Np + J * T + c];
        a[r][c] = S[(size_t)(I * T + r) * Np + K * T + c];
    }
    __syncthreads();
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int r = e / T, c = e % T;
        double s = a[r][c];
        for (int k = 0; k < T; ++k) s = fma(-li[r][k], lk[c][k], s);
        a[r][c] = s;
    }
    if (I == K && threadIdx.x < T) {
        const int r = threadIdx.x;
        double s = rhs[I * T + r];
        for (int k = 0; k < T; ++k) s = fma(-li[r][k], rhs[J * T + k], s);
        b[r] = s;
    }
    __syncthreads();
    if (I == K && I == J + 1) {
        if (!tile_potrf(a, linv, b, y, status)) return;
        tile_store_diag(a, linv, y, I, Np, S, Linv, rhs);
        return;
    }
    for (int e = threadIdx.x; e < TT; e += blockDim.x) {
        const int r = e / T, c = e % T;
        S[(size_t)(I * T + r) * Np + K * T + c] = a[r][c];
    }
    if (I == K && threadIdx.x < T) rhs[I * T + threadIdx.x] = b[threadIdx.x];
}

// Back solve step J (descending): x_J = Linv_J^T y_J; tiles I < J update
// y_I -= L_JI^T x_J.  One block per I in [0, J].
__global__ void __launch_bounds__(TT) k_chol_back(int J, int Np, const double *S, const double *Linv,
                                                  double *rhs, double *x, const int *status)
{
    if (*status) return;
    __shared__ double xj[T];
    const int I = blockIdx.x;
    if (threadIdx.x < T) {
        const int c = threadIdx.x;
        double s = 0.0;
        for (int k = c; k < T; ++k) s = fma(Linv[(size_t)J * TT + k * T + c], rhs[J * T + k], s);
        xj[c] = s;
    }
    __syncthreads();
    if (I == J) {
        if (threadIdx.x < T) x[J * T + threadIdx.x] = xj[threadIdx.x];
        return;
    }
    if (threadIdx.x < T) {
        const int r = threadIdx.x;
        double s = rhs[I * T + r];
        for (int c = 0; c < T; ++c) s = fma(-S[(size_t)(J * T + c) * Np + I * T + r], xj[c], s);
        rhs[I * T + r] = s;
    }
}

void launch_cholesky_solve(const DeviceProblem &d, cudaStream_t s)
{
    const int nb = d.Np / T;
    k_chol_first<<<1, TT, 0, s>>>(d.Np, d.S, d.Linv, d.rhs, d.status); note_launch(1);
    for (int J = 0; J + 1 < nb; ++J) {
        k_chol_trsm<<<nb - J - 1, TT, 0, s>>>(J, d.Np, d.S, d.Linv, d.status); note_launch(1);
        const int m = nb - J - 1;
        k_chol_update<<<m * (m + 1) / 2, TT, 0, s>>>(J, nb, d.Np, d.S, d.Linv, d.rhs, d.status); note_launch(1);
    }
    for (int J = nb - 1; J >= 0; --J)
        k_chol_back<<<J + 1, TT, 0, s>>>(J, d.Np, d.S, d.Linv, d.rhs, d.xsol, d.status); note_launch(1);
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

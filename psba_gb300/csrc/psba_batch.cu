// Batched solver: many independent small problems in one persistent launch.
//
// Each CTA takes a problem index from a device queue (one atomic counter),
// runs that problem's whole Levenberg-Marquardt solve -- the control flow of
// levmar() (PSBA/levmar.cpp:45-256) with every stage of the reference's
// kernel chain done by the CTA's threads -- writes its result and takes the
// next problem.  CTAs never wait for each other, and a problem's arithmetic
// does not depend on which CTA runs it or what else is in the batch, so a
// problem gives the same bits alone and inside any batch.
//
// Per-problem layout: one table entry (BatchProblem) with element offsets into
// three arenas (double, int, and R = double or float for the per-observation
// arrays).  Stages inside a CTA:
//   camera tables, residual/Jacobian/W per observation (threads over obs),
//   V and gb per point (threads over points), U and ga per camera and the
//   Schur blocks (one warp per camera / per camera pair, lanes over the
//   entries, fixed-order shuffle reductions), V^-1 and Y, the FP64 Cholesky of
//   S and both triangular solves (CTA, column by column), eb/dpb, the trial
//   cost and the LM decision (thread 0).
// The shape parameters -- threads per CTA and, per problem, lanes per camera
// pair in the Schur stage -- are chosen per size bucket by the autotuner in
// psba_gb300/batch.py.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "psba_batch_internal.h"

namespace psba {
namespace batch {

constexpr int MAX_THREADS = 512;

// ---------------------------------------------------------------- helpers

__device__ __forceinline__ double cta_sum(double v, double *sh)
{
    // fixed-order tree over the CTA (blockDim.x a power of two <= MAX_THREADS)
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) sh[threadIdx.x] += sh[threadIdx.x + st];
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__device__ __forceinline__ double cta_max(double v, double *sh)
{
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int st = blockDim.x / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) sh[threadIdx.x] = fmax(sh[threadIdx.x], sh[threadIdx.x + st]);
        __syncthreads();
    }
    const double r = sh[0];
    __syncthreads();
    return r;
}

__device__ __forceinline__ double warp_sum(double v)
{
    for (int off = 16; off > 0; off >>= 1) v += __shfl_down_sync(0xffffffffu, v, off);
    return v;  // lane 0 holds the fixed-order sum
}

// camera table: rotation q(v) (x) q0 as a matrix, its derivative w.r.t. v,
// translation and intrinsics (same content as k_cam_tables)
__device__ void cam_table(const double *K, const double *q0, const double *cam, const double *dpa, double *o)
{
    double vl[3], t[3];
    for (int m = 0; m < 3; ++m) {
        vl[m] = dpa ? cam[m] + dpa[m] : cam[m];
        t[m] = dpa ? cam[3 + m] + dpa[3 + m] : cam[3 + m];
    }
    const double s0 = q0[0], a1 = q0[1], a2 = q0[2], a3 = q0[3];
    const double sl = sqrt(1.0 - vl[0] * vl[0] - vl[1] * vl[1] - vl[2] * vl[2]);
    const double s = sl * s0 - (a1 * vl[0] + a2 * vl[1] + a3 * vl[2]);
    const double a = s0 * vl[0] + sl * a1 + a3 * vl[1] - a2 * vl[2];
    const double b = s0 * vl[1] + sl * a2 + a1 * vl[2] - a3 * vl[0];
    const double c = s0 * vl[2] + sl * a3 + a2 * vl[0] - a1 * vl[1];
    const double d = s * s - (a * a + b * b + c * c);
    o[0] = d + 2 * a * a;       o[1] = 2 * (a * b - s * c); o[2] = 2 * (a * c + s * b);
    o[3] = 2 * (a * b + s * c); o[4] = d + 2 * b * b;       o[5] = 2 * (b * c - s * a);
    o[6] = 2 * (a * c - s * b); o[7] = 2 * (b * c + s * a); o[8] = d + 2 * c * c;
    const double dS[9] = {2 * s, -2 * c, 2 * b, 2 * c, 2 * s, -2 * a, -2 * b, 2 * a, 2 * s};
    const double dA[9] = {2 * a, 2 * b, 2 * c, 2 * b, -2 * a, -2 * s, 2 * c, 2 * s, -2 * a};
    const double dB[9] = {-2 * b, 2 * a, 2 * s, 2 * a, 2 * b, 2 * c, -2 * s, 2 * c, -2 * b};
    const double dC[9] = {-2 * c, -2 * s, 2 * a, 2 * s, -2 * c, 2 * b, 2 * a, 2 * b, 2 * c};
    const double av[3] = {a1, a2, a3};
    for (int m = 0; m < 3; ++m) {
        const double ds = -vl[m] / sl;
        double e_x_a[3] = {0, 0, 0};
        if (m == 0) { e_x_a[1] = -a3; e_x_a[2] = a2; }
        if (m == 1) { e_x_a[0] = a3; e_x_a[2] = -a1; }
        if (m == 2) { e_x_a[0] = -a2; e_x_a[1] = a1; }
        const double dq0 = s0 * ds - av[m];
        double dqv[3];
        for (int r = 0; r < 3; ++r) dqv[r] = av[r] * ds + (r == m ? s0 : 0.0) + e_x_a[r];
        for (int e = 0; e < 9; ++e) o[9 + 9 * m + e] = dS[e] * dq0 + dA[e] * dqv[0] + dB[e] * dqv[1] + dC[e] * dqv[2];
    }
    o[36] = t[0]; o[37] = t[1]; o[38] = t[2];
    o[39] = K[0]; o[40] = K[4]; o[41] = K[1]; o[42] = K[0] * K[3]; o[43] = K[2];
}

// squared residual of one observation at (table, point)
__device__ __forceinline__ double obs_sq(const double *T, const double X0, const double X1, const double X2,
                                         const double *m)
{
    const double xc = T[0] * X0 + T[1] * X1 + T[2] * X2 + T[36];
    const double yc = T[3] * X0 + T[4] * X1 + T[5] * X2 + T[37];
    const double zc = T[6] * X0 + T[7] * X1 + T[8] * X2 + T[38];
    const double iz = 1.0 / zc;
    const double u = (T[39] * xc + T[40] * yc + T[41] * zc) * iz;
    const double v = (T[42] * yc + T[43] * zc) * iz;
    const double e0 = m[0] - u, e1 = m[1] - v;
    return e0 * e0 + e1 * e1;
}

template <typename R> struct Arenas {
    double *d;
    int *i;
    R *r;
};

// ---------------------------------------------------------------- stages

template <typename R>
__device__ double stage_cost(const BatchProblem &p, const Arenas<R> &ar, const double *tab, const double *dpb,
                             double *sh)
{
    const int *opt = ar.i + p.i_obs_pt, *ocam = ar.i + p.i_obs_cam;
    const double *pts = ar.d + p.d_pts, *meas = ar.d + p.d_meas;
    double acc = 0.0;
    for (int o = threadIdx.x; o < p.no; o += blockDim.x) {
        const int i = opt[o], j = ocam[o];
        double X0 = pts[3 * i], X1 = pts[3 * i + 1], X2 = pts[3 * i + 2];
        if (dpb) {
            X0 = X0 + dpb[3 * i];
            X1 = X1 + dpb[3 * i + 1];
            X2 = X2 + dpb[3 * i + 2];
        }
        acc += obs_sq(tab + (size_t)CAMTAB * j, X0, X1, X2, meas + 2 * (size_t)o);
    }
    return cta_sum(acc, sh);
}

template <typename R>
__device__ void stage_tables(const BatchProblem &p, const Arenas<R> &ar, const double *dpa, double *tab)
{
    for (int j = threadIdx.x; j < p.nc; j += blockDim.x)
        cam_table(ar.d + p.d_K + 5 * j, ar.d + p.d_q0 + 4 * j, ar.d + p.d_cams + 6 * j, dpa ? dpa + 6 * j : nullptr,
                  tab + (size_t)CAMTAB * j);
}

template <typename R>
__device__ void stage_linearize(const BatchProblem &p, const Arenas<R> &ar)
{
    const int *opt = ar.i + p.i_obs_pt, *ocam = ar.i + p.i_obs_cam;
    const double *pts = ar.d + p.d_pts, *meas = ar.d + p.d_meas, *tab = ar.d + p.d_tab;
    R *ex = ar.r + p.r_ex, *A = ar.r + p.r_A, *B = ar.r + p.r_B, *W = ar.r + p.r_W;
    for (int o = threadIdx.x; o < p.no; o += blockDim.x) {
        const int i = opt[o], j = ocam[o];
        const double *T = tab + (size_t)CAMTAB * j;
        // projection and residual in FP64 in both forms; only the stored e, J, W are R
        const double Xd0 = pts[3 * i], Xd1 = pts[3 * i + 1], Xd2 = pts[3 * i + 2];
        const double xcd = T[0] * Xd0 + T[1] * Xd1 + T[2] * Xd2 + T[36];
        const double ycd = T[3] * Xd0 + T[4] * Xd1 + T[5] * Xd2 + T[37];
        const double zcd = T[6] * Xd0 + T[7] * Xd1 + T[8] * Xd2 + T[38];
        const double izd = 1.0 / zcd;
        const double nud = T[39] * xcd + T[40] * ycd;
        ex[2 * (size_t)o] = (R)(meas[2 * (size_t)o] - (nud + T[41] * zcd) * izd);
        ex[2 * (size_t)o + 1] = (R)(meas[2 * (size_t)o + 1] - (T[42] * ycd + T[43] * zcd) * izd);
        const R X0 = (R)Xd0, X1 = (R)Xd1, X2 = (R)Xd2;
        R M[9];
        for (int e = 0; e < 9; ++e) M[e] = (R)T[e];
        const R yc = (R)ycd, iz = (R)izd, nu = (R)nud, fx = (R)T[39], sk = (R)T[40], fy = (R)T[42];
        const R p00 = fx * iz, p01 = sk * iz, p02 = -nu * iz * iz, p11 = fy * iz, p12 = -fy * yc * iz * iz;
        R a[12], bb[6];
        for (int m = 0; m < 3; ++m) {
            const double *Dm = T + 9 + 9 * m;
            const R g0 = (R)Dm[0] * X0 + (R)Dm[1] * X1 + (R)Dm[2] * X2;
            const R g1 = (R)Dm[3] * X0 + (R)Dm[4] * X1 + (R)Dm[5] * X2;
            const R g2 = (R)Dm[6] * X0 + (R)Dm[7] * X1 + (R)Dm[8] * X2;
            a[m] = p00 * g0 + p01 * g1 + p02 * g2;
            a[6 + m] = p11 * g1 + p12 * g2;
            bb[m] = p00 * M[m] + p01 * M[3 + m] + p02 * M[6 + m];
            bb[3 + m] = p11 * M[3 + m] + p12 * M[6 + m];
        }
        a[3] = p00; a[4] = p01; a[5] = p02;
        a[9] = (R)0; a[10] = p11; a[11] = p12;
        R *Ao = A + 12 * (size_t)o, *Bo = B + 6 * (size_t)o, *Wo = W + 18 * (size_t)o;
        for (int e = 0; e < 12; ++e) Ao[e] = a[e];
        for (int e = 0; e < 6; ++e) Bo[e] = bb[e];
        for (int r = 0; r < 6; ++r)
            for (int c = 0; c < 3; ++c) Wo[r * 3 + c] = a[r] * bb[c] + a[6 + r] * bb[3 + c];
    }
}

template <typename R>
__device__ void stage_points(const BatchProblem &p, const Arenas<R> &ar)
{
    const int *ps = ar.i + p.i_pt_start;
    const R *B = ar.r + p.r_B, *ex = ar.r + p.r_ex;
    double *V = ar.d + p.d_V, *g = ar.d + p.d_g, *uvd = ar.d + p.d_uvdiag;
    for (int i = threadIdx.x; i < p.np; i += blockDim.x) {
        double v[6] = {0, 0, 0, 0, 0, 0};
        double g0 = 0, g1 = 0, g2 = 0;
        for (int o = ps[i]; o < ps[i + 1]; ++o) {
            const R *b = B + 6 * (size_t)o;
            const R e0 = ex[2 * (size_t)o], e1 = ex[2 * (size_t)o + 1];
            v[0] += (double)(b[0] * b[0] + b[3] * b[3]);
            v[1] += (double)(b[0] * b[1] + b[3] * b[4]);
            v[2] += (double)(b[0] * b[2] + b[3] * b[5]);
            v[3] += (double)(b[1] * b[1] + b[4] * b[4]);
            v[4] += (double)(b[1] * b[2] + b[4] * b[5]);
            v[5] += (double)(b[2] * b[2] + b[5] * b[5]);
            g0 = g0 + (double)b[0] * (double)e0 + (double)b[3] * (double)e1;
            g1 = g1 + (double)b[1] * (double)e0 + (double)b[4] * (double)e1;
            g2 = g2 + (double)b[2] * (double)e0 + (double)b[5] * (double)e1;
        }
        for (int e = 0; e < 6; ++e) V[6 * (size_t)i + e] = v[e];
        uvd[p.N + 3 * i] = v[0];
        uvd[p.N + 3 * i + 1] = v[3];
        uvd[p.N + 3 * i + 2] = v[5];
        g[p.N + 3 * i] = g0;
        g[p.N + 3 * i + 1] = g1;
        g[p.N + 3 * i + 2] = g2;
    }
}

// U and ga, one warp per camera, lanes strided over the camera's observations
template <typename R>
__device__ void stage_cameras(const BatchProblem &p, const Arenas<R> &ar)
{
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
    const int *cs = ar.i + p.i_cam_start, *co = ar.i + p.i_cam_obs;
    const R *A = ar.r + p.r_A, *ex = ar.r + p.r_ex;
    double *U = ar.d + p.d_U, *g = ar.d + p.d_g, *uvd = ar.d + p.d_uvdiag;
    for (int j = warp; j < p.nc; j += nw) {
        double acc[27];
        for (int v = 0; v < 27; ++v) acc[v] = 0.0;
        for (int t = cs[j] + lane; t < cs[j + 1]; t += 32) {
            const int o = co[t];
            const R *a = A + 12 * (size_t)o;
            const R e0 = ex[2 * (size_t)o], e1 = ex[2 * (size_t)o + 1];
            int v = 0;
            for (int r = 0; r < 6; ++r)
                for (int c = r; c < 6; ++c, ++v) acc[v] += (double)(a[r] * a[c] + a[6 + r] * a[6 + c]);
            for (int k = 0; k < 6; ++k) acc[21 + k] += (double)a[k] * (double)e0 + (double)a[6 + k] * (double)e1;
        }
        for (int v = 0; v < 27; ++v) acc[v] = warp_sum(acc[v]);
        if (lane == 0) {
            int v = 0;
            for (int r = 0; r < 6; ++r)
                for (int c = r; c < 6; ++c, ++v) {
                    U[36 * j + r * 6 + c] = acc[v];
                    U[36 * j + c * 6 + r] = acc[v];
                    if (r == c) uvd[6 * j + r] = acc[v];
                }
            for (int k = 0; k < 6; ++k) g[6 * j + k] = acc[21 + k];
        }
    }
}

__device__ void vinv3(const double *Vi, double mu, double *out)
{
    const double a11 = Vi[0] + mu, a12 = Vi[1], a13 = Vi[2], a22 = Vi[3] + mu, a23 = Vi[4], a33 = Vi[5] + mu;
    double T = (a33 * a12 * a12 - 2 * a12 * a13 * a23 + a22 * a13 * a13 + a11 * a23 * a23 - a11 * a22 * a33);
    if (fabs(T) < 1e-16) {
        const double a21 = a12, a31 = a13, a32 = a23;
        double m[3][3] = {{a11, a12, a13}, {a21, a22, a23}, {a31, a32, a33}}, tmp;
        int mx = 0;
        if (m[0][0] < m[1][0]) mx = 1;
        if (m[mx][0] < m[2][0]) mx = 2;
        if (mx != 0)
            for (int c = 0; c < 3; ++c) { tmp = m[0][c]; m[0][c] = m[mx][c]; m[mx][c] = tmp; }
        m[1][0] = m[1][0] / m[0][0];
        m[2][0] = m[2][0] / m[0][0];
        m[1][1] = m[1][1] - m[1][0] * m[0][1];
        m[1][2] = m[1][2] - m[1][0] * m[0][2];
        m[2][1] = m[2][1] - m[2][0] * m[0][1];
        m[2][2] = m[2][2] - m[2][0] * m[0][2];
        if (m[1][1] < m[2][1])
            for (int c = 0; c < 3; ++c) { tmp = m[1][c]; m[1][c] = m[2][c]; m[2][c] = tmp; }
        if (m[1][1] != 0.0) {
            m[2][1] = m[2][1] / m[1][1];
            m[2][2] = m[2][2] - m[2][1] * m[1][2];
        }
        T = m[0][0] * m[1][1] * m[2][2];
        out[0] = (a22 * a33 - a23 * a32) / T;
        out[1] = -(a21 * a33 - a23 * a31) / T;
        out[2] = (a21 * a32 - a22 * a31) / T;
        out[3] = (a11 * a33 - a13 * a31) / T;
        out[4] = -(a11 * a32 - a12 * a31) / T;
        out[5] = (a11 * a22 - a12 * a21) / T;
        return;
    }
    out[0] = -(-a23 * a23 + a22 * a33) / T;
    out[1] = -(a13 * a23 - a12 * a33) / T;
    out[2] = -(a12 * a23 - a13 * a22) / T;
    out[3] = -(-a13 * a13 + a11 * a33) / T;
    out[4] = -(a12 * a13 - a11 * a23) / T;
    out[5] = -(-a12 * a12 + a11 * a22) / T;
}

template <typename R>
__device__ void stage_vinv_y(const BatchProblem &p, const Arenas<R> &ar, double mu)
{
    const double *V = ar.d + p.d_V;
    double *Vi = ar.d + p.d_Vinv;
    for (int i = threadIdx.x; i < p.np; i += blockDim.x) vinv3(V + 6 * (size_t)i, mu, Vi + 6 * (size_t)i);
    __syncthreads();
    const int *opt = ar.i + p.i_obs_pt;
    const R *W = ar.r + p.r_W;
    R *Y = ar.r + p.r_Y;
    for (int o = threadIdx.x; o < p.no; o += blockDim.x) {
        const double *s = Vi + 6 * (size_t)opt[o];
        const R *w = W + 18 * (size_t)o;
        R *y = Y + 18 * (size_t)o;
        for (int r = 0; r < 6; ++r) {
            const double w0 = w[3 * r], w1 = w[3 * r + 1], w2 = w[3 * r + 2];
            y[3 * r] = (R)(w0 * s[0] + w1 * s[1] + w2 * s[2]);
            y[3 * r + 1] = (R)(w0 * s[1] + w1 * s[3] + w2 * s[4]);
            y[3 * r + 2] = (R)(w0 * s[2] + w1 * s[4] + w2 * s[5]);
        }
    }
}

// S (N x N, row-major, lower triangle) and rhs = ea
template <typename R>
__device__ void stage_schur(const BatchProblem &p, const Arenas<R> &ar, double mu)
{
    const int N = p.N;
    double *S = ar.d + p.d_S, *rhs = ar.d + p.d_rhs;
    for (long long e = threadIdx.x; e < (long long)N * N; e += blockDim.x) S[e] = 0.0;
    __syncthreads();
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
    const R *Y = ar.r + p.r_Y, *W = ar.r + p.r_W;
    const double *U = ar.d + p.d_U, *g = ar.d + p.d_g;
    const int *opt = ar.i + p.i_obs_pt, *cs = ar.i + p.i_cam_start, *co = ar.i + p.i_cam_obs;
    // diagonal blocks and ea
    for (int k = warp; k < p.nc; k += nw) {
        double acc[27];
        for (int v = 0; v < 27; ++v) acc[v] = 0.0;
        for (int t = cs[k] + lane; t < cs[k + 1]; t += 32) {
            const int a = co[t];
            const R *y = Y + 18 * (size_t)a, *w = W + 18 * (size_t)a;
            const double *gb = g + N + 3 * (size_t)opt[a];
            int v = 0;
            for (int r = 0; r < 6; ++r)
                for (int c = 0; c <= r; ++c, ++v)
                    acc[v] += (double)(y[3 * r] * w[3 * c] + y[3 * r + 1] * w[3 * c + 1] + y[3 * r + 2] * w[3 * c + 2]);
            for (int r = 0; r < 6; ++r)
                acc[21 + r] += (double)y[3 * r] * gb[0] + (double)y[3 * r + 1] * gb[1] + (double)y[3 * r + 2] * gb[2];
        }
        for (int v = 0; v < 27; ++v) acc[v] = warp_sum(acc[v]);
        if (lane == 0) {
            int v = 0;
            for (int r = 0; r < 6; ++r)
                for (int c = 0; c <= r; ++c, ++v) {
                    const double uu = U[36 * k + r * 6 + c];
                    S[(size_t)(6 * k + r) * N + 6 * k + c] = (r == c ? uu + mu : uu) - acc[v];
                }
            for (int r = 0; r < 6; ++r) rhs[6 * k + r] = g[6 * k + r] - acc[21 + r];
        }
    }
    // off-diagonal blocks: groups of `lpp` lanes per camera pair (8, 16 or 32,
    // the autotuner's choice for the problem's size bucket), lanes strided
    // over the pair's common points, fixed-order shuffle reduction
    const int *pst = ar.i + p.i_pair_start, *pkl = ar.i + p.i_pair_kl, *pa = ar.i + p.i_pair_a,
              *pb = ar.i + p.i_pair_b;
    const int lpp = (p.flags & 0xff) ? (p.flags & 0xff) : 32;
    const int gpw = 32 / lpp;                       // groups per warp
    const int grp = warp * gpw + lane / lpp, ng = nw * gpw, gl = lane % lpp;
    const int qmax = (p.n_pairs + ng - 1) / ng * ng;  // keep whole warps in the loop for the shuffles
    for (int q = grp; q < qmax; q += ng) {
        double acc[36];
        for (int v = 0; v < 36; ++v) acc[v] = 0.0;
        if (q < p.n_pairs) {
            for (int t = pst[q] + gl; t < pst[q + 1]; t += lpp) {
                const R *y = Y + 18 * (size_t)pa[t], *w = W + 18 * (size_t)pb[t];
                for (int r = 0; r < 6; ++r)
                    for (int c = 0; c < 6; ++c)
                        acc[r * 6 + c] +=
                            (double)(y[3 * r] * w[3 * c] + y[3 * r + 1] * w[3 * c + 1] + y[3 * r + 2] * w[3 * c + 2]);
            }
        }
        for (int v = 0; v < 36; ++v)
            for (int off = lpp / 2; off > 0; off >>= 1) acc[v] += __shfl_down_sync(0xffffffffu, acc[v], off, lpp);
        if (gl == 0 && q < p.n_pairs) {
            const int k = pkl[2 * q], l = pkl[2 * q + 1];
            for (int r = 0; r < 6; ++r)
                for (int c = 0; c < 6; ++c) S[(size_t)(6 * k + r) * N + 6 * l + c] = -acc[r * 6 + c];
        }
    }
}

// Right-looking column Cholesky of the lower triangle of S (FP64), then
// L y = rhs and L^T x = y.  Returns 0, or 1 on a non-positive / non-finite
// pivot (the reference's status, SPD_inv.cl:66-107).
__device__ int stage_cholesky_solve(double *S, int N, double *rhs, double *x, double *sh, int *shi)
{
    if (threadIdx.x == 0) shi[0] = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int k = 0; k < N; ++k) {
        if (threadIdx.x == 0) {
            const double d = S[(size_t)k * N + k];
            if (!(d > 0.0) || !isfinite(d)) {
                shi[0] = 1;
            } else {
                // one root on the column chain: L_kk = d / sqrt(d); the forward
                // solve rides along (y_k = rhs_k / L_kk), and 1 / L_kk waits in
                // x[k] for the back solve
                const double r = rsqrt(d);
                S[(size_t)k * N + k] = d * r;
                const double yk = rhs[k] * r;
                rhs[k] = yk;
                x[k] = r;
                sh[0] = r;
                sh[1] = yk;
            }
        }
        __syncthreads();
        if (shi[0]) return 1;
        const double inv = sh[0], yk = sh[1];
        for (int i = k + 1 + threadIdx.x; i < N; i += blockDim.x) {
            const double l = S[(size_t)i * N + k] * inv;
            S[(size_t)i * N + k] = l;
            rhs[i] -= l * yk;
        }
        __syncthreads();
        // trailing update, lower triangle: a warp per row, lanes over its columns
        for (int i = k + 1 + warp; i < N; i += nwarps) {
            const double lik = S[(size_t)i * N + k];
            for (int j = k + 1 + lane; j <= i; j += 32) S[(size_t)i * N + j] -= lik * S[(size_t)j * N + k];
        }
        __syncthreads();
    }
    // back: L^T x = y (y in rhs, 1 / L_kk in x[k])
    for (int k = N - 1; k >= 0; --k) {
        if (threadIdx.x == 0) x[k] = rhs[k] * x[k];
        __syncthreads();
        const double xk = x[k];
        for (int i = threadIdx.x; i < k; i += blockDim.x) rhs[i] -= S[(size_t)k * N + i] * xk;
        __syncthreads();
    }
    return 0;
}

// eb, dpb into dp[N..]; returns (|dp|^2, dp.(mu dp + g)) through sh2
template <typename R>
__device__ void stage_back(const BatchProblem &p, const Arenas<R> &ar, double mu, double *sh, double out[2])
{
    const int N = p.N;
    double *dp = ar.d + p.d_dp;
    const double *g = ar.d + p.d_g, *Vi = ar.d + p.d_Vinv;
    const int *ps = ar.i + p.i_pt_start, *ocam = ar.i + p.i_obs_cam;
    const R *W = ar.r + p.r_W;
    double s_sq = 0.0, s_rho = 0.0;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        const double x = dp[k];
        s_sq += x * x;
        s_rho += x * (mu * x + g[k]);
    }
    for (int i = threadIdx.x; i < p.np; i += blockDim.x) {
        double e0 = 0, e1 = 0, e2 = 0;
        for (int o = ps[i]; o < ps[i + 1]; ++o) {
            const R *w = W + 18 * (size_t)o;
            const double *da = dp + 6 * (size_t)ocam[o];
            for (int k = 0; k < 6; ++k) {
                e0 += (double)w[3 * k] * da[k];
                e1 += (double)w[3 * k + 1] * da[k];
                e2 += (double)w[3 * k + 2] * da[k];
            }
        }
        const double *gb = g + N + 3 * (size_t)i;
        e0 = gb[0] - e0;
        e1 = gb[1] - e1;
        e2 = gb[2] - e2;
        const double *v = Vi + 6 * (size_t)i;
        const double d0 = v[0] * e0 + v[1] * e1 + v[2] * e2;
        const double d1 = v[1] * e0 + v[3] * e1 + v[4] * e2;
        const double d2 = v[2] * e0 + v[4] * e1 + v[5] * e2;
        double *db = dp + N + 3 * (size_t)i;
        db[0] = d0;
        db[1] = d1;
        db[2] = d2;
        s_sq += d0 * d0 + d1 * d1 + d2 * d2;
        s_rho += d0 * (mu * d0 + gb[0]) + d1 * (mu * d1 + gb[1]) + d2 * (mu * d2 + gb[2]);
    }
    out[0] = cta_sum(s_sq, sh);
    out[1] = cta_sum(s_rho, sh);
}

// ---------------------------------------------------------------- mixed form
// The mixed form's stages (R = float): no FP64 instruction per observation,
// as in the single-problem kernels.  On GB300 a conversion between FP32 and
// FP64 issues on the FP64 pipe, so FP32 products added into FP64 sums cost
// the FP64 rate per term; instead the sums are double-float (two FP32 values
// hi + lo, TwoSum, ~2^-44 of the terms) or FP32 chains of at most eight
// observations flushed into double-float, converted to FP64 once per output.
// The projections (linearization, trial cost) run in double-float from the
// camera tables, points and measurements split into FP32 pairs once; Y takes
// V^-1 split once per point; eb takes the camera step split once.

__device__ __forceinline__ float2 *rf2(const Arenas<float> &ar, long long off)
{
    return reinterpret_cast<float2 *>(ar.r + off);
}

// vector loads and stores of FP32 rows (8-byte aligned: every R-arena region
// offset is even; A's rows 16-byte aligned)
__device__ __forceinline__ void ld2n(const float *p, float *out, int n)
{
    const float2 *q = reinterpret_cast<const float2 *>(p);
    for (int k = 0; k < n / 2; ++k) {
        const float2 v = q[k];
        out[2 * k] = v.x;
        out[2 * k + 1] = v.y;
    }
}
__device__ __forceinline__ void st2n(float *p, const float *in, int n)
{
    float2 *q = reinterpret_cast<float2 *>(p);
    for (int k = 0; k < n / 2; ++k) q[k] = make_float2(in[2 * k], in[2 * k + 1]);
}
// nine consecutive floats of a 72-byte row starting at float 9 h (h = 0, 1):
// four 8-byte pairs and one scalar
__device__ __forceinline__ void ld_half9(const float *row, int h, float (&v)[9])
{
    const float *p = row + 9 * h;
    const float single = p[h ? 0 : 8];
    const float2 *q = reinterpret_cast<const float2 *>(p + (h ? 1 : 0));
    float pr[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 t = q[k];
        pr[2 * k] = t.x;
        pr[2 * k + 1] = t.y;
    }
    v[0] = h ? single : pr[0];
#pragma unroll
    for (int e = 1; e < 8; ++e) v[e] = h ? pr[e - 1] : pr[e];
    v[8] = h ? pr[7] : single;
}

// df accumulator: h + l += x (x an FP32 value)
__device__ __forceinline__ void dacc(float &h, float &l, float x)
{
    float t;
    two_sum_f(h, x, h, t);
    l += t;
}

// fixed-order df sum over a warp (shuffle-down tree, as warp_sum): lane 0
__device__ __forceinline__ void warp_sum_df(float &h, float &l)
{
    for (int off = 16; off > 0; off >>= 1) {
        const float oh = __shfl_down_sync(0xffffffffu, h, off), ol = __shfl_down_sync(0xffffffffu, l, off);
        float t;
        two_sum_f(h, oh, h, t);
        l += ol + t;
    }
}

// camera tables plus the FP32 Jacobian copy (tab32, optional) and the
// projection's FP32-pair split (tab2f)
__device__ void stage_tables_mx(const BatchProblem &p, const Arenas<float> &ar, const double *dpa, double *tab,
                                float *tab32, float2 *tab2f)
{
    for (int j = threadIdx.x; j < p.nc; j += blockDim.x) {
        double *o = tab + (size_t)CAMTAB * j;
        cam_table(ar.d + p.d_K + 5 * j, ar.d + p.d_q0 + 4 * j, ar.d + p.d_cams + 6 * j, dpa ? dpa + 6 * j : nullptr,
                  o);
        if (tab32) {
            float *F = tab32 + (size_t)CAMTAB32 * j;
            for (int e = 0; e < 36; ++e) F[e] = (float)o[e];
            F[36] = (float)o[39];
            F[37] = (float)o[40];
            F[38] = (float)o[42];
            F[39] = 0.0f;
        }
        float2 *F2 = tab2f + (size_t)RES_TAB2F * j;
        for (int e = 0; e < 9; ++e) F2[e] = split2f(o[e]);
        for (int e = 0; e < 3; ++e) F2[9 + e] = split2f(o[36 + e]);
        for (int e = 0; e < 5; ++e) F2[12 + e] = split2f(o[39 + e]);  // fx sk cx fy cy
        F2[17] = make_float2(0.0f, 0.0f);
    }
}

// one observation's residual in double-float: m - pi(X) at a split table row
__device__ __forceinline__ void proj_df(const float2 *T, df X0, df X1, df X2, float4 m, df &e0, df &e1, df &ycv,
                                        df &izv, df &nuv)
{
    const df xc = df_add(df_add(df_mul(df_of(T[0]), X0), df_mul(df_of(T[1]), X1)),
                         df_add(df_mul(df_of(T[2]), X2), df_of(T[9])));
    ycv = df_add(df_add(df_mul(df_of(T[3]), X0), df_mul(df_of(T[4]), X1)), df_add(df_mul(df_of(T[5]), X2), df_of(T[10])));
    const df zc = df_add(df_add(df_mul(df_of(T[6]), X0), df_mul(df_of(T[7]), X1)),
                         df_add(df_mul(df_of(T[8]), X2), df_of(T[11])));
    izv = df_rcp(zc);
    nuv = df_add(df_mul(df_of(T[12]), xc), df_mul(df_of(T[13]), ycv));
    const df un = df_add(nuv, df_mul(df_of(T[14]), zc));
    const df vn = df_add(df_mul(df_of(T[15]), ycv), df_mul(df_of(T[16]), zc));
    e0 = df_add(df{m.x, m.y}, df_neg(df_mul(un, izv)));
    e1 = df_add(df{m.z, m.w}, df_neg(df_mul(vn, izv)));
}

// the measurements (once per launch) or the current points split into pairs
__device__ void split_into(const double *x, float2 *out, long long n)
{
    for (long long k = threadIdx.x; k < n; k += blockDim.x) out[k] = split2f(x[k]);
}

__device__ void stage_linearize_mx(const BatchProblem &p, const Arenas<float> &ar)
{
    const int *opt = ar.i + p.i_obs_pt, *ocam = ar.i + p.i_obs_cam;
    const float2 *T2 = rf2(ar, p.r_tab2f), *X2 = rf2(ar, p.r_pts2f);
    const float4 *M4 = reinterpret_cast<const float4 *>(ar.r + p.r_meas2f);
    const float *T32 = ar.r + p.r_tab32;
    float *ex = ar.r + p.r_ex, *A = ar.r + p.r_A, *B = ar.r + p.r_B, *W = ar.r + p.r_W;
    for (int o = threadIdx.x; o < p.no; o += blockDim.x) {
        const int i = opt[o], j = ocam[o];
        const df Xa = df_of(X2[3 * i]), Xb = df_of(X2[3 * i + 1]), Xc = df_of(X2[3 * i + 2]);
        df e0, e1, ycv, izv, nuv;
        proj_df(T2 + (size_t)RES_TAB2F * j, Xa, Xb, Xc, M4[o], e0, e1, ycv, izv, nuv);
        *reinterpret_cast<float2 *>(ex + 2 * (size_t)o) = make_float2(__fadd_rn(e0.hi, e0.lo), __fadd_rn(e1.hi, e1.lo));
        const float X0 = Xa.hi, X1 = Xb.hi, X2v = Xc.hi;
        const float yc = __fadd_rn(ycv.hi, ycv.lo), iz = __fadd_rn(izv.hi, izv.lo), nu = __fadd_rn(nuv.hi, nuv.lo);
        const float *F = T32 + (size_t)CAMTAB32 * j;
        const float fx = F[36], sk = F[37], fy = F[38];
        const float p00 = fx * iz, p01 = sk * iz, p02 = -nu * iz * iz, p11 = fy * iz, p12 = -fy * yc * iz * iz;
        float a[12], bb[6];
        for (int m = 0; m < 3; ++m) {
            const float *Dm = F + 9 + 9 * m;
            const float g0 = Dm[0] * X0 + Dm[1] * X1 + Dm[2] * X2v;
            const float g1 = Dm[3] * X0 + Dm[4] * X1 + Dm[5] * X2v;
            const float g2 = Dm[6] * X0 + Dm[7] * X1 + Dm[8] * X2v;
            a[m] = p00 * g0 + p01 * g1 + p02 * g2;
            a[6 + m] = p11 * g1 + p12 * g2;
            bb[m] = p00 * F[m] + p01 * F[3 + m] + p02 * F[6 + m];
            bb[3 + m] = p11 * F[3 + m] + p12 * F[6 + m];
        }
        a[3] = p00; a[4] = p01; a[5] = p02;
        a[9] = 0.0f; a[10] = p11; a[11] = p12;
        float4 *A4 = reinterpret_cast<float4 *>(A + 12 * (size_t)o);
#pragma unroll
        for (int k = 0; k < 3; ++k) A4[k] = make_float4(a[4 * k], a[4 * k + 1], a[4 * k + 2], a[4 * k + 3]);
        st2n(B + 6 * (size_t)o, bb, 6);
        float wv[18];
#pragma unroll
        for (int r = 0; r < 6; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) wv[r * 3 + c] = a[r] * bb[c] + a[6 + r] * bb[3 + c];
        st2n(W + 18 * (size_t)o, wv, 18);
    }
}

// V and gb per point: the FP32 products of V and the exact products of gb
// in double-float, one conversion per value (gb also rounded to FP32 for the
// ea sums)
__device__ void stage_points_mx(const BatchProblem &p, const Arenas<float> &ar)
{
    const int *ps = ar.i + p.i_pt_start;
    const float *B = ar.r + p.r_B, *ex = ar.r + p.r_ex;
    double *V = ar.d + p.d_V, *g = ar.d + p.d_g, *uvd = ar.d + p.d_uvdiag;
    float *gb32 = ar.r + p.r_gb32;
    for (int i = threadIdx.x; i < p.np; i += blockDim.x) {
        float h[9], l[9];
        for (int v = 0; v < 9; ++v) h[v] = l[v] = 0.0f;
        for (int o = ps[i]; o < ps[i + 1]; ++o) {
            float b[6];
            ld2n(B + 6 * (size_t)o, b, 6);
            const float2 ee = *reinterpret_cast<const float2 *>(ex + 2 * (size_t)o);
            const float e0 = ee.x, e1 = ee.y;
            dacc(h[0], l[0], fmaf(b[0], b[0], b[3] * b[3]));
            dacc(h[1], l[1], fmaf(b[0], b[1], b[3] * b[4]));
            dacc(h[2], l[2], fmaf(b[0], b[2], b[3] * b[5]));
            dacc(h[3], l[3], fmaf(b[1], b[1], b[4] * b[4]));
            dacc(h[4], l[4], fmaf(b[1], b[2], b[4] * b[5]));
            dacc(h[5], l[5], fmaf(b[2], b[2], b[5] * b[5]));
            for (int k = 0; k < 3; ++k) {
                const float p0 = __fmul_rn(b[k], e0), p1 = __fmul_rn(b[3 + k], e1);
                const float q = fmaf(b[k], e0, -p0) + fmaf(b[3 + k], e1, -p1);
                float t0, t1;
                two_sum_f(h[6 + k], p0, h[6 + k], t0);
                two_sum_f(h[6 + k], p1, h[6 + k], t1);
                l[6 + k] += (t0 + t1) + q;
            }
        }
        for (int e = 0; e < 6; ++e) V[6 * (size_t)i + e] = (double)h[e] + (double)l[e];
        uvd[p.N + 3 * i] = V[6 * (size_t)i];
        uvd[p.N + 3 * i + 1] = V[6 * (size_t)i + 3];
        uvd[p.N + 3 * i + 2] = V[6 * (size_t)i + 5];
        for (int k = 0; k < 3; ++k) {
            g[p.N + 3 * i + k] = (double)h[6 + k] + (double)l[6 + k];
            gb32[4 * i + k] = __fadd_rn(h[6 + k], l[6 + k]);
        }
    }
}

// xor-tree df sum over the lanes of equal lane & 3 (offsets 4, 8, 16):
// lanes 0..3 hold the totals
__device__ __forceinline__ void slot_sum_df(float &h, float &l)
{
    for (int off = 4; off < 32; off <<= 1) {
        const float oh = __shfl_xor_sync(0xffffffffu, h, off), ol = __shfl_xor_sync(0xffffffffu, l, off);
        float t;
        two_sum_f(h, oh, h, t);
        l += ol + t;
    }
}

// U and ga, one warp per camera: lane 4 s + q takes the camera's
// observations s, s + 8, ... and quadrant q of U (q = 0: rows and columns
// 0-2; 1: rows 0-2, columns 3-5; 3: rows and columns 3-5) or, for q = 2, the
// six sums of ga.  U's FP32 products are summed over eight of the lane's
// observations at a time, then into double-float; ga's exact products in
// double-float; the eight slots meet in a fixed xor tree.
__device__ void stage_cameras_mx(const BatchProblem &p, const Arenas<float> &ar)
{
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
    const int q = lane & 3, s = lane >> 2, r0 = q == 3 ? 3 : 0, c0 = q == 0 ? 0 : 3;
    const int *cs = ar.i + p.i_cam_start, *co = ar.i + p.i_cam_obs;
    const float *A = ar.r + p.r_A, *ex = ar.r + p.r_ex;
    double *U = ar.d + p.d_U, *g = ar.d + p.d_g, *uvd = ar.d + p.d_uvdiag;
    for (int j = warp; j < p.nc; j += nw) {
        float h[9], l[9], part[9];
#pragma unroll
        for (int v = 0; v < 9; ++v) h[v] = l[v] = part[v] = 0.0f;
        int n = 0;
        for (int t = cs[j] + s; t < cs[j + 1]; t += 8) {
            const int o = co[t];
            float a[12];
            const float4 *A4 = reinterpret_cast<const float4 *>(A + 12 * (size_t)o);
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                const float4 x = A4[k];
                a[4 * k] = x.x;
                a[4 * k + 1] = x.y;
                a[4 * k + 2] = x.z;
                a[4 * k + 3] = x.w;
            }
            if (q == 2) {
                const float2 ee = *reinterpret_cast<const float2 *>(ex + 2 * (size_t)o);
                const float e0 = ee.x, e1 = ee.y;
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const float p0 = __fmul_rn(a[k], e0), p1 = __fmul_rn(a[6 + k], e1);
                    const float qq = fmaf(a[k], e0, -p0) + fmaf(a[6 + k], e1, -p1);
                    float t0, t1;
                    two_sum_f(h[k], p0, h[k], t0);
                    two_sum_f(h[k], p1, h[k], t1);
                    l[k] += (t0 + t1) + qq;
                }
            } else {
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c)
                        part[3 * r + c] = part[3 * r + c] + a[r0 + r] * a[c0 + c] + a[6 + r0 + r] * a[6 + c0 + c];
                if (++n == 8) {
#pragma unroll
                    for (int v = 0; v < 9; ++v) {
                        dacc(h[v], l[v], part[v]);
                        part[v] = 0.0f;
                    }
                    n = 0;
                }
            }
        }
#pragma unroll
        for (int v = 0; v < 9; ++v) {
            dacc(h[v], l[v], part[v]);
            slot_sum_df(h[v], l[v]);
        }
        if (s == 0) {
            if (q == 2) {
#pragma unroll
                for (int k = 0; k < 6; ++k) g[6 * j + k] = (double)h[k] + (double)l[k];
            } else {
#pragma unroll
                for (int r = 0; r < 3; ++r)
#pragma unroll
                    for (int c = 0; c < 3; ++c) {
                        const int R = r0 + r, C = c0 + c;
                        if (R > C) continue;  // the upper triangle, mirrored
                        const double x = (double)h[3 * r + c] + (double)l[3 * r + c];
                        U[36 * j + R * 6 + C] = x;
                        U[36 * j + C * 6 + R] = x;
                        if (R == C) uvd[6 * j + R] = x;
                    }
            }
        }
    }
}

// V^-1 in FP64 per point (split once into pairs), then Y = W V^-1 in
// double-float per observation
__device__ void stage_vinv_y_mx(const BatchProblem &p, const Arenas<float> &ar, double mu)
{
    const double *V = ar.d + p.d_V;
    double *Vi = ar.d + p.d_Vinv;
    float2 *vs = rf2(ar, p.r_vinv2f);
    for (int i = threadIdx.x; i < p.np; i += blockDim.x) {
        double out[6];
        vinv3(V + 6 * (size_t)i, mu, out);
        for (int e = 0; e < 6; ++e) {
            Vi[6 * (size_t)i + e] = out[e];
            vs[6 * (size_t)i + e] = split2f(out[e]);
        }
    }
    __syncthreads();
    const int *opt = ar.i + p.i_obs_pt;
    const float *W = ar.r + p.r_W;
    float *Y = ar.r + p.r_Y;
    for (int o = threadIdx.x; o < p.no; o += blockDim.x) {
        const float2 *s = vs + 6 * (size_t)opt[o];
        const float2 s00 = s[0], s01 = s[1], s02 = s[2], s11 = s[3], s12 = s[4], s22 = s[5];
        float w[18], y[18];
        ld2n(W + 18 * (size_t)o, w, 18);
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            const float w0 = w[3 * r], w1 = w[3 * r + 1], w2 = w[3 * r + 2];
            y[3 * r] = dot3_df(w0, w1, w2, s00, s01, s02);
            y[3 * r + 1] = dot3_df(w0, w1, w2, s01, s11, s12);
            y[3 * r + 2] = dot3_df(w0, w1, w2, s02, s12, s22);
        }
        st2n(Y + 18 * (size_t)o, y, 18);
    }
}

// S and ea.  Diagonal blocks: a warp per camera, lanes strided over its
// observations, FP32 products (ea with gb in FP32) over eight observations
// at a time, then double-float.  Off-diagonal blocks: lpp lanes per camera
// pair, lane 4 s + q on quadrant q of the 6 x 6 block (rows 3 (q >> 1) ..,
// columns 3 (q & 1) ..) and on the pair's common points s, s + lpp / 4, ...,
// FP32 over eight of them at a time, then double-float, the slots combined
// by a fixed xor tree.
__device__ void stage_schur_mx(const BatchProblem &p, const Arenas<float> &ar, double mu)
{
    const int N = p.N;
    double *S = ar.d + p.d_S, *rhs = ar.d + p.d_rhs;
    for (long long e = threadIdx.x; e < (long long)N * N; e += blockDim.x) S[e] = 0.0;
    __syncthreads();
    const int warp = threadIdx.x / 32, lane = threadIdx.x % 32, nw = blockDim.x / 32;
    const float *Y = ar.r + p.r_Y, *W = ar.r + p.r_W, *gb32 = ar.r + p.r_gb32;
    const double *U = ar.d + p.d_U, *g = ar.d + p.d_g;
    const int *opt = ar.i + p.i_obs_pt, *cs = ar.i + p.i_cam_start, *co = ar.i + p.i_cam_obs;
    {
        // diagonal blocks: lane 4 s + q on the camera's observations s, s + 8,
        // ... and quadrant q of the lower block (0: rows and columns 0-2; 2:
        // rows 3-5, columns 0-2; 3: rows and columns 3-5) or, for q = 1, the
        // six ea sums
        const int qd = lane & 3, sd = lane >> 2, r0 = qd >= 2 ? 3 : 0, c0 = qd == 3 ? 3 : 0;
        for (int k = warp; k < p.nc; k += nw) {
            float h[9], l[9], part[9];
#pragma unroll
            for (int v = 0; v < 9; ++v) h[v] = l[v] = part[v] = 0.0f;
            int n = 0;
            for (int t = cs[k] + sd; t < cs[k + 1]; t += 8) {
                const int a = co[t];
                const float *y = Y + 18 * (size_t)a, *w = W + 18 * (size_t)a;
                if (qd == 1) {
                    const float4 gb = *reinterpret_cast<const float4 *>(gb32 + 4 * (size_t)opt[a]);
                    const float g0 = gb.x, g1 = gb.y, g2 = gb.z;
                    float yr[18];
                    ld2n(y, yr, 18);
#pragma unroll
                    for (int r = 0; r < 6; ++r) {
                        float sm = part[r];
                        sm = fmaf(yr[3 * r], g0, sm);
                        sm = fmaf(yr[3 * r + 1], g1, sm);
                        sm = fmaf(yr[3 * r + 2], g2, sm);
                        part[r] = sm;
                    }
                } else {
                    float yv[9], wv[9];
                    ld_half9(y, r0 / 3, yv);
                    ld_half9(w, c0 / 3, wv);
#pragma unroll
                    for (int r = 0; r < 3; ++r)
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            float sm = part[3 * r + c];
                            sm = fmaf(yv[3 * r], wv[3 * c], sm);
                            sm = fmaf(yv[3 * r + 1], wv[3 * c + 1], sm);
                            sm = fmaf(yv[3 * r + 2], wv[3 * c + 2], sm);
                            part[3 * r + c] = sm;
                        }
                }
                if (++n == 8) {
#pragma unroll
                    for (int v = 0; v < 9; ++v) {
                        dacc(h[v], l[v], part[v]);
                        part[v] = 0.0f;
                    }
                    n = 0;
                }
            }
#pragma unroll
            for (int v = 0; v < 9; ++v) {
                dacc(h[v], l[v], part[v]);
                slot_sum_df(h[v], l[v]);
            }
            if (sd == 0) {
                if (qd == 1) {
#pragma unroll
                    for (int r = 0; r < 6; ++r) rhs[6 * k + r] = g[6 * k + r] - ((double)h[r] + (double)l[r]);
                } else {
#pragma unroll
                    for (int r = 0; r < 3; ++r)
#pragma unroll
                        for (int c = 0; c < 3; ++c) {
                            const int R = r0 + r, C = c0 + c;
                            if (C > R) continue;  // the lower triangle
                            const double uu = U[36 * k + R * 6 + C];
                            S[(size_t)(6 * k + R) * N + 6 * k + C] =
                                (R == C ? uu + mu : uu) - ((double)h[3 * r + c] + (double)l[3 * r + c]);
                        }
                }
            }
        }
    }
    const int *pst = ar.i + p.i_pair_start, *pkl = ar.i + p.i_pair_kl, *pa = ar.i + p.i_pair_a,
              *pb = ar.i + p.i_pair_b;
    const int lpp = (p.flags & 0xff) ? (p.flags & 0xff) : 32;  // 8, 16 or 32
    const int gpw = 32 / lpp, grp = warp * gpw + lane / lpp, ng = nw * gpw, gl = lane % lpp;
    const int q4 = gl & 3, s4 = gl >> 2, nslot = lpp >> 2, qr = q4 >> 1, qc = q4 & 1;
    const int qmax = (p.n_pairs + ng - 1) / ng * ng;  // keep whole warps in the loop for the shuffles
    for (int q = grp; q < qmax; q += ng) {
        float h[9], l[9], part[9];
        for (int v = 0; v < 9; ++v) h[v] = l[v] = part[v] = 0.0f;
        if (q < p.n_pairs) {
            int n = 0;
            for (int t = pst[q] + s4; t < pst[q + 1]; t += nslot) {
                float yv[9], wv[9];
                ld_half9(Y + 18 * (size_t)pa[t], qr, yv);
                ld_half9(W + 18 * (size_t)pb[t], qc, wv);
                for (int r = 0; r < 3; ++r)
                    for (int c = 0; c < 3; ++c) {
                        float sm = part[3 * r + c];
                        sm = fmaf(yv[3 * r], wv[3 * c], sm);
                        sm = fmaf(yv[3 * r + 1], wv[3 * c + 1], sm);
                        sm = fmaf(yv[3 * r + 2], wv[3 * c + 2], sm);
                        part[3 * r + c] = sm;
                    }
                if (++n == 8) {
                    for (int v = 0; v < 9; ++v) {
                        dacc(h[v], l[v], part[v]);
                        part[v] = 0.0f;
                    }
                    n = 0;
                }
            }
            for (int v = 0; v < 9; ++v) dacc(h[v], l[v], part[v]);
        }
        for (int v = 0; v < 9; ++v)
            for (int off = 4; off < lpp; off <<= 1) {
                const float oh = __shfl_xor_sync(0xffffffffu, h[v], off), ol = __shfl_xor_sync(0xffffffffu, l[v], off);
                float t;
                two_sum_f(h[v], oh, h[v], t);
                l[v] += ol + t;
            }
        if (s4 == 0 && q < p.n_pairs) {
            const int k = pkl[2 * q], l2 = pkl[2 * q + 1];
            for (int r = 0; r < 3; ++r)
                for (int c = 0; c < 3; ++c)
                    S[(size_t)(6 * k + 3 * qr + r) * N + 6 * l2 + 3 * qc + c] =
                        -((double)h[3 * r + c] + (double)l[3 * r + c]);
        }
    }
}

// eb = gb - W^T dpa in double-float (dpa split once), dpb = V^-1 eb in
// FP64 per point; the trial points split for the trial cost
__device__ void stage_back_mx(const BatchProblem &p, const Arenas<float> &ar, double mu, double *sh, double out[2])
{
    const int N = p.N;
    double *dp = ar.d + p.d_dp;
    const double *g = ar.d + p.d_g, *Vi = ar.d + p.d_Vinv, *pts = ar.d + p.d_pts;
    const int *ps = ar.i + p.i_pt_start, *ocam = ar.i + p.i_obs_cam;
    const float *W = ar.r + p.r_W;
    float2 *da2 = rf2(ar, p.r_dpa2f), *x2 = rf2(ar, p.r_x2f);
    double s_sq = 0.0, s_rho = 0.0;
    for (int k = threadIdx.x; k < N; k += blockDim.x) {
        const double x = dp[k];
        da2[k] = split2f(x);
        s_sq += x * x;
        s_rho += x * (mu * x + g[k]);
    }
    __syncthreads();
    for (int i = threadIdx.x; i < p.np; i += blockDim.x) {
        float h[3] = {0.0f, 0.0f, 0.0f}, l[3] = {0.0f, 0.0f, 0.0f};
        for (int o = ps[i]; o < ps[i + 1]; ++o) {
            float w[18];
            ld2n(W + 18 * (size_t)o, w, 18);
            const float2 *da = da2 + 6 * (size_t)ocam[o];
            for (int k = 0; k < 6; ++k) {
                const float2 d2 = da[k];
                for (int c = 0; c < 3; ++c) {
                    const float wv = w[3 * k + c];
                    const float pr = __fmul_rn(wv, d2.x);
                    const float pe = fmaf(wv, d2.x, -pr);
                    float t;
                    two_sum_f(h[c], pr, h[c], t);
                    l[c] = fmaf(wv, d2.y, l[c] + (t + pe));
                }
            }
        }
        const double *gb = g + N + 3 * (size_t)i;
        const double e0 = gb[0] - ((double)h[0] + (double)l[0]);
        const double e1 = gb[1] - ((double)h[1] + (double)l[1]);
        const double e2 = gb[2] - ((double)h[2] + (double)l[2]);
        const double *v = Vi + 6 * (size_t)i;
        const double d0 = v[0] * e0 + v[1] * e1 + v[2] * e2;
        const double d1 = v[1] * e0 + v[3] * e1 + v[4] * e2;
        const double d2 = v[2] * e0 + v[4] * e1 + v[5] * e2;
        double *db = dp + N + 3 * (size_t)i;
        db[0] = d0;
        db[1] = d1;
        db[2] = d2;
        x2[3 * (size_t)i] = split2f(pts[3 * (size_t)i] + d0);
        x2[3 * (size_t)i + 1] = split2f(pts[3 * (size_t)i + 1] + d1);
        x2[3 * (size_t)i + 2] = split2f(pts[3 * (size_t)i + 2] + d2);
        s_sq += d0 * d0 + d1 * d1 + d2 * d2;
        s_rho += d0 * (mu * d0 + gb[0]) + d1 * (mu * d1 + gb[1]) + d2 * (mu * d2 + gb[2]);
    }
    out[0] = cta_sum(s_sq, sh);
    out[1] = cta_sum(s_rho, sh);
}

// the trial cost in double-float: the trial table's split and the trial
// points' (stage_back_mx), the measurements' pairs
__device__ double stage_cost_mx(const BatchProblem &p, const Arenas<float> &ar, double *sh)
{
    const int *opt = ar.i + p.i_obs_pt, *ocam = ar.i + p.i_obs_cam;
    const float2 *T2 = rf2(ar, p.r_tab2f2), *X2 = rf2(ar, p.r_x2f);
    const float4 *M4 = reinterpret_cast<const float4 *>(ar.r + p.r_meas2f);
    df sq{0.0f, 0.0f};
    for (int o = threadIdx.x; o < p.no; o += blockDim.x) {
        const int i = opt[o], j = ocam[o];
        df e0, e1, ycv, izv, nuv;
        proj_df(T2 + (size_t)RES_TAB2F * j, df_of(X2[3 * i]), df_of(X2[3 * i + 1]), df_of(X2[3 * i + 2]), M4[o], e0,
                e1, ycv, izv, nuv);
        sq = df_add(sq, df_add(df_mul(e0, e0), df_mul(e1, e1)));
    }
    return cta_sum((double)sq.hi + (double)sq.lo, sh);
}

// ---------------------------------------------------------------- one problem

template <typename R>
__device__ void solve_problem(const BatchProblem &p, const Arenas<R> &ar, const BatchOpts &o, BatchResult *res,
                              double *sh, int *shi, double *shd)
{
    const int N = p.N;
    double *dp = ar.d + p.d_dp, *tab = ar.d + p.d_tab, *tab2 = ar.d + p.d_tab2;
    double *cams = ar.d + p.d_cams, *pts = ar.d + p.d_pts;
    // shd: 0 mu, 1 p_L2, 2 ex_L2, 3 new cost; shi: 1 iter_flag, 2 nu, 3 itno, 4 trials, 5 lin, 6 first, 7 loop
    if (!res->started) {
        stage_tables<R>(p, ar, nullptr, tab);
        __syncthreads();
        const double c0 = stage_cost<R>(p, ar, tab, nullptr, sh);
        if (threadIdx.x == 0) {
            shd[0] = 0.0;
            shd[1] = 0.0;
            shd[2] = c0;
            shi[1] = PSBA_ITER_CONTINUE;
            shi[2] = 2;
            shi[3] = 0;
            shi[4] = 0;
            shi[5] = 0;
            shi[6] = 1;
            res->initial_cost = c0;
        }
    } else if (threadIdx.x == 0) {
        shd[0] = res->mu;
        shd[1] = res->p_L2;
        shd[2] = res->final_cost;
        shi[1] = res->status;
        shi[2] = res->nu;
        shi[3] = res->iterations;
        shi[4] = res->trials;
        shi[5] = res->linearizations;
        shi[6] = res->first;
    }
    __syncthreads();
    constexpr bool MX = sizeof(R) == 4;  // the mixed form
    if constexpr (MX) split_into(ar.d + p.d_meas, rf2(ar, p.r_meas2f), 2LL * p.no);
    const int slice_end = p.slice > 0 ? shi[3] + p.slice : o.max_iter;
    while (shi[3] < o.max_iter && shi[3] < slice_end && shi[1] == PSBA_ITER_CONTINUE) {
        if constexpr (MX) {
            stage_tables_mx(p, ar, nullptr, tab, ar.r + p.r_tab32, rf2(ar, p.r_tab2f));
            split_into(pts, rf2(ar, p.r_pts2f), 3LL * p.np);
            __syncthreads();
            stage_linearize_mx(p, ar);
            __syncthreads();
            stage_points_mx(p, ar);
            stage_cameras_mx(p, ar);
        } else {
            stage_tables<R>(p, ar, nullptr, tab);
            __syncthreads();
            stage_linearize<R>(p, ar);
            __syncthreads();
            stage_points<R>(p, ar);
            stage_cameras<R>(p, ar);
        }
        __syncthreads();
        if (threadIdx.x == 0) shi[5]++;
        if (shi[6]) {
            const double *uvd = ar.d + p.d_uvdiag;
            double m = 0.0;
            for (int k = threadIdx.x; k < N + 3 * p.np; k += blockDim.x) m = fmax(m, uvd[k]);
            m = cta_max(m, sh);
            if (threadIdx.x == 0) {
                shd[0] = o.tau * m;
                shd[1] = 1e+3;
                shi[2] = 2;
                shi[6] = 0;
            }
            __syncthreads();
        }
        while (true) {
            const double mu = shd[0];
            if constexpr (MX) {
                stage_vinv_y_mx(p, ar, mu);
                __syncthreads();
                stage_schur_mx(p, ar, mu);
            } else {
                stage_vinv_y<R>(p, ar, mu);
                __syncthreads();
                stage_schur<R>(p, ar, mu);
            }
            __syncthreads();
            double *S = ar.d + p.d_S, *rhs = ar.d + p.d_rhs, *x = ar.d + p.d_x;
            const int st = stage_cholesky_solve(S, N, rhs, x, sh, shi);
            if (threadIdx.x == 0) shi[4]++;
            int decided = 0;  // 0: retry with larger mu, 1: accepted, 2: stop
            if (st == 0) {
                for (int k = threadIdx.x; k < N; k += blockDim.x) dp[k] = x[k];
                __syncthreads();
                double sums[2];
                if constexpr (MX)
                    stage_back_mx(p, ar, mu, sh, sums);
                else
                    stage_back<R>(p, ar, mu, sh, sums);
                const double dp_L2 = sums[0], rho_den = sums[1];
                if (dp_L2 < shd[1] * o.stop_thresh * o.stop_thresh) {
                    if (threadIdx.x == 0) shi[1] = PSBA_ITER_DP_NO_CHANGE;
                    decided = 2;
                } else if (dp_L2 >= (shd[1] + o.stop_thresh) / (o.eps * o.eps)) {
                    if (threadIdx.x == 0) shi[1] = PSBA_ITER_ERR;
                    decided = 2;
                } else {
                    double new_cost;
                    if constexpr (MX) {
                        stage_tables_mx(p, ar, dp, tab2, nullptr, rf2(ar, p.r_tab2f2));
                        __syncthreads();
                        new_cost = stage_cost_mx(p, ar, sh);
                    } else {
                        stage_tables<R>(p, ar, dp, tab2);
                        __syncthreads();
                        new_cost = stage_cost<R>(p, ar, tab2, dp + N, sh);
                    }
                    const double rho = (shd[2] - new_cost) / rho_den;
                    if (rho > 0) {
                        for (int k = threadIdx.x; k < N; k += blockDim.x) cams[k] = cams[k] + dp[k];
                        for (int k = threadIdx.x; k < 3 * p.np; k += blockDim.x) pts[k] = pts[k] + dp[N + k];
                        __syncthreads();
                        double a = 0.0;
                        for (int k = threadIdx.x; k < N; k += blockDim.x) a += cams[k] * cams[k];
                        const double pa = cta_sum(a, sh);
                        double b = 0.0;
                        for (int k = threadIdx.x; k < 3 * p.np; k += blockDim.x) b += pts[k] * pts[k];
                        const double pb = cta_sum(b, sh);
                        if (threadIdx.x == 0) {
                            double tmp = 2 * rho - 1;
                            tmp = 1.0 - tmp * tmp * tmp;
                            shd[0] = mu * ((tmp >= (1.0 / 3.0)) ? tmp : (1.0 / 3.0));
                            shi[2] = 2;
                            shd[1] = pa + pb;
                            shd[2] = new_cost;
                        }
                        decided = 1;
                    }
                }
            }
            __syncthreads();
            if (decided == 2) break;
            if (decided == 1) break;
            if (threadIdx.x == 0) {
                shd[0] = shd[0] * shi[2];
                const int nu2 = (int)(2u * (unsigned)shi[2]);
                if (nu2 <= shi[2]) shi[1] = PSBA_ITER_ERR;
                shi[2] = nu2;
            }
            __syncthreads();
            if (shi[1] != PSBA_ITER_CONTINUE) break;
        }
        if (threadIdx.x == 0) {
            if (shd[2] <= o.stop_thresh) shi[1] = PSBA_ITER_ERR_SMALL_ENOUGH;
            shi[3]++;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        res->status = shi[1];
        res->iterations = shi[3];
        res->trials = shi[4];
        res->linearizations = shi[5];
        res->final_cost = shd[2];
        res->mu = shd[0];
        res->p_L2 = shd[1];
        res->nu = shi[2];
        res->first = shi[6];
        res->started = 1;
    }
    __syncthreads();
}

template <typename R>
__global__ void __launch_bounds__(MAX_THREADS) k_batch_lm(const BatchProblem *__restrict__ probs,
                                                           const int *__restrict__ order, int n,
                                                           int *__restrict__ queue, Arenas<R> ar,
                                                           const BatchOpts *__restrict__ opts,
                                                           BatchResult *__restrict__ res)
{
    const BatchOpts o = *opts;
    __shared__ double sh[MAX_THREADS];
    __shared__ double shd[8];
    __shared__ int shi[16];
    __shared__ int next;
    while (true) {
        if (threadIdx.x == 0) next = atomicAdd(queue, 1);
        __syncthreads();
        const int q = next;
        __syncthreads();
        if (q >= n) break;
        const int pi = order[q];
        const BatchProblem p = probs[pi];
        solve_problem<R>(p, ar, o, res + pi, sh, shi, shd);
    }
}

// ---------------------------------------------------------------- host side

bool build_problem_layout(const psba_problem_desc &p, ProblemLayout &L, std::string &err)
{
    if (p.cnp != 0 && p.cnp != 6) {
        err = "the batched engine takes 6-parameter cameras (cnp 0 or 6)";
        return false;
    }
    if (p.cov) {
        err = "the batched engine takes unweighted problems (cov must be NULL)";
        return false;
    }
    if (p.n_cams <= 0 || p.n_pts < 0 || p.n_obs < 0 || !p.K || !p.q0 || !p.cams || (p.n_pts && !p.pts) ||
        (p.n_obs && (!p.meas || !p.obs_pt || !p.obs_cam))) {
        err = "problem is malformed";
        return false;
    }
    for (int o = 0; o < p.n_obs; ++o) {
        const int i = p.obs_pt[o], j = p.obs_cam[o];
        bool bad = i < 0 || i >= p.n_pts || j < 0 || j >= p.n_cams;
        if (!bad && o > 0) bad = i < p.obs_pt[o - 1] || (i == p.obs_pt[o - 1] && j <= p.obs_cam[o - 1]);
        if (bad) {
            err = "observations out of range or not sorted by (point, camera)";
            return false;
        }
    }
    BatchProblem &bp = L.bp;
    std::memset(&bp, 0, sizeof(bp));
    std::vector<double> &dA = L.dA;
    std::vector<int> &iA = L.iA;
    dA.clear();
    iA.clear();
    const int nc = p.n_cams, np = p.n_pts, no = p.n_obs, N = 6 * nc;
    bp.nc = nc;
    bp.np = np;
    bp.no = no;
    bp.N = N;
    auto dput = [&](const double *src, size_t cnt) {
        const long long at = (long long)dA.size();
        dA.insert(dA.end(), src, src + cnt);
        return at;
    };
    auto dres = [&](size_t cnt) {
        const long long at = (long long)dA.size();
        dA.resize(dA.size() + cnt, 0.0);
        return at;
    };
    auto iput = [&](const int *src, size_t cnt) {
        const long long at = (long long)iA.size();
        iA.insert(iA.end(), src, src + cnt);
        return at;
    };
    bp.d_K = dput(p.K, 5 * (size_t)nc);
    bp.d_q0 = dput(p.q0, 4 * (size_t)nc);
    bp.d_cams = dput(p.cams, 6 * (size_t)nc);
    bp.d_pts = dput(p.pts, 3 * (size_t)np);
    bp.d_cams0 = dput(p.cams, 6 * (size_t)nc);
    bp.d_pts0 = dput(p.pts, 3 * (size_t)np);
    bp.d_meas = dput(p.meas, 2 * (size_t)no);
    bp.i_obs_pt = iput(p.obs_pt, no);
    bp.i_obs_cam = iput(p.obs_cam, no);
    std::vector<int> ps(np + 1, 0), cs(nc + 1, 0), co(no);
    for (int o = 0; o < no; ++o) {
        ps[p.obs_pt[o] + 1]++;
        cs[p.obs_cam[o] + 1]++;
    }
    for (int i = 0; i < np; ++i) ps[i + 1] += ps[i];
    for (int j = 0; j < nc; ++j) cs[j + 1] += cs[j];
    {
        std::vector<int> fill(cs.begin(), cs.end() - 1);
        for (int o = 0; o < no; ++o) co[fill[p.obs_cam[o]]++] = o;
    }
    bp.i_pt_start = iput(ps.data(), ps.size());
    bp.i_cam_start = iput(cs.data(), cs.size());
    bp.i_cam_obs = iput(co.data(), co.size());
    std::vector<int> id((size_t)nc * nc, -1), kl, cnt;
    for (int i = 0; i < np; ++i)
        for (int a = ps[i]; a < ps[i + 1]; ++a)
            for (int c = ps[i]; c < a; ++c) {
                int &x = id[(size_t)p.obs_cam[a] * nc + p.obs_cam[c]];
                if (x < 0) {
                    x = (int)cnt.size();
                    kl.push_back(p.obs_cam[a]);
                    kl.push_back(p.obs_cam[c]);
                    cnt.push_back(0);
                }
                cnt[x]++;
            }
    const int npair = (int)cnt.size();
    std::vector<int> pst(npair + 1, 0);
    for (int x = 0; x < npair; ++x) pst[x + 1] = pst[x] + cnt[x];
    std::vector<int> pa(pst[npair]), pb(pst[npair]);
    {
        std::vector<int> fill(pst.begin(), pst.end() - 1);
        for (int i = 0; i < np; ++i)
            for (int a = ps[i]; a < ps[i + 1]; ++a)
                for (int c = ps[i]; c < a; ++c) {
                    const int x = id[(size_t)p.obs_cam[a] * nc + p.obs_cam[c]];
                    pa[fill[x]] = a;
                    pb[fill[x]++] = c;
                }
    }
    bp.n_pairs = npair;
    bp.i_pair_start = iput(pst.data(), pst.size());
    bp.i_pair_kl = iput(kl.data(), kl.size());
    bp.i_pair_a = iput(pa.data(), pa.size());
    bp.i_pair_b = iput(pb.data(), pb.size());
    long long r_total = 0;
    // A first: its 48-byte rows stay 16-byte aligned (every region and the
    // problem's total are multiples of four elements), the others 8-byte
    bp.r_A = r_total; r_total += 12LL * no;
    bp.r_W = r_total; r_total += 18LL * no;
    bp.r_Y = r_total; r_total += 18LL * no;
    bp.r_B = r_total; r_total += 6LL * no;
    bp.r_ex = r_total; r_total += 2LL * no;
    // the mixed form's FP32 copies (even counts: FP32 pairs stay 8-byte aligned)
    bp.r_tab32 = r_total; r_total += (long long)CAMTAB32 * nc;
    bp.r_tab2f = r_total; r_total += 2LL * RES_TAB2F * nc;
    bp.r_tab2f2 = r_total; r_total += 2LL * RES_TAB2F * nc;
    bp.r_meas2f = r_total; r_total += 4LL * no;
    bp.r_pts2f = r_total; r_total += 6LL * np;
    bp.r_x2f = r_total; r_total += 6LL * np;
    bp.r_vinv2f = r_total; r_total += 12LL * np;
    bp.r_dpa2f = r_total; r_total += 2LL * N;
    bp.r_gb32 = r_total; r_total += 4LL * np;
    L.nr = r_total;
    bp.d_V = dres(6 * (size_t)np);
    bp.d_Vinv = dres(6 * (size_t)np);
    bp.d_U = dres(36 * (size_t)nc);
    bp.d_g = dres((size_t)N + 3 * (size_t)np);
    bp.d_uvdiag = dres((size_t)N + 3 * (size_t)np);
    bp.d_dp = dres((size_t)N + 3 * (size_t)np);
    bp.d_S = dres((size_t)N * N);
    bp.d_tab = dres((size_t)CAMTAB * nc);
    bp.d_tab2 = dres((size_t)CAMTAB * nc);
    bp.d_rhs = dres((size_t)N);
    bp.d_x = dres((size_t)N);
    // one LM iteration: per-observation work plus the in-CTA FP64 Cholesky
    L.work = (double)no + 0.02 * std::pow((double)N, 3) / 64.0;
    return true;
}

void rebase_problem(BatchProblem &bp, long long db, long long ib, long long rb)
{
    for (long long *f : {&bp.d_K, &bp.d_q0, &bp.d_cams, &bp.d_pts, &bp.d_cams0, &bp.d_pts0, &bp.d_meas, &bp.d_V,
                         &bp.d_Vinv, &bp.d_U, &bp.d_g, &bp.d_uvdiag, &bp.d_dp, &bp.d_S, &bp.d_tab,
                         &bp.d_tab2, &bp.d_rhs, &bp.d_x})
        *f += db;
    for (long long *f : {&bp.i_obs_pt, &bp.i_obs_cam, &bp.i_pt_start, &bp.i_cam_start, &bp.i_cam_obs,
                         &bp.i_pair_start, &bp.i_pair_kl, &bp.i_pair_a, &bp.i_pair_b})
        *f += ib;
    for (long long *f : {&bp.r_ex, &bp.r_A, &bp.r_B, &bp.r_W, &bp.r_Y, &bp.r_tab32, &bp.r_tab2f, &bp.r_tab2f2,
                         &bp.r_meas2f, &bp.r_pts2f, &bp.r_x2f, &bp.r_vinv2f, &bp.r_dpa2f, &bp.r_gb32})
        *f += rb;
}

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

size_t pool_bytes(const ProblemLayout &L, int precision)
{
    const size_t rs = precision == PSBA_PREC_MIXED ? sizeof(float) : sizeof(double);
    return align256(sizeof(double) * L.dA.size()) + align256(sizeof(int) * L.iA.size()) + align256(rs * L.nr);
}

cudaError_t launch_batch_lm(int precision, int grid, int threads, cudaStream_t s, const BatchProblem *probs,
                            const int *order, int n, int *queue, double *darena, int *iarena, void *rarena,
                            const BatchOpts *opts, BatchResult *res)
{
    if (precision == PSBA_PREC_MIXED) {
        Arenas<float> ar{darena, iarena, (float *)rarena};
        k_batch_lm<float><<<grid, threads, 0, s>>>(probs, order, n, queue, ar, opts, res);
    } else {
        Arenas<double> ar{darena, iarena, (double *)rarena};
        k_batch_lm<double><<<grid, threads, 0, s>>>(probs, order, n, queue, ar, opts, res);
    }
    return cudaGetLastError();  // the caller counts the launch (it may be inside a graph capture)
}

int batch_blocks_per_sm(int precision, int threads)
{
    int per_sm = 1;
    if (precision == PSBA_PREC_MIXED)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_lm<float>, threads, 0);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch_lm<double>, threads, 0);
    return per_sm > 0 ? per_sm : 1;
}


struct HostBatch {
    int n = 0;
    std::vector<BatchProblem> probs;
    std::vector<int> order;
    BatchProblem *d_probs = nullptr;
    int *d_order = nullptr, *d_queue = nullptr;
    double *d_arena = nullptr;
    int *i_arena = nullptr;
    void *r_arena = nullptr;  // sized for double
    long long nd = 0, ni = 0, nr = 0;
    BatchResult *d_res = nullptr;
    BatchOpts *d_opts = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    int threads = 256;
    size_t bytes = 0;
    cudaGraphExec_t graph = nullptr;  // captured [queue reset, persistent launch]
    int graph_key = -1;               // precision * 1024 + threads of the captured graph
};

}  // namespace batch
}  // namespace psba

using namespace psba;
using namespace psba::batch;

struct psba_batch {
    HostBatch hb;
};

namespace {

int cuda_fail(cudaError_t e, const char *what)
{
    set_error(std::string(what) + ": " + cudaGetErrorString(e));
    return PSBA_ERR_CUDA;
}

void batch_free(psba_batch *b)
{
    if (!b) return;
    HostBatch &h = b->hb;
    if (h.stream) cudaStreamSynchronize(h.stream);
    cudaFree(h.d_probs);
    cudaFree(h.d_order);
    cudaFree(h.d_queue);
    cudaFree(h.d_arena);
    cudaFree(h.i_arena);
    cudaFree(h.r_arena);
    cudaFree(h.d_res);
    cudaFree(h.d_opts);
    if (h.graph) cudaGraphExecDestroy(h.graph);
    if (h.ev0) cudaEventDestroy(h.ev0);
    if (h.ev1) cudaEventDestroy(h.ev1);
    if (h.stream) cudaStreamDestroy(h.stream);
    delete b;
}

}  // namespace

extern "C" {

int psba_batch_create(const psba_problem_desc *descs, int n, psba_batch **out)
{
    if (!out || !descs || n <= 0) return set_error("psba_batch_create: bad arguments"), PSBA_ERR_ARG;
    *out = nullptr;
    psba_batch *b = new psba_batch();
    HostBatch &h = b->hb;
    h.n = n;
    h.probs.resize(n);
    // host layouts, concatenated into the three arenas
    std::vector<double> dA;
    std::vector<int> iA;
    long long r_total = 0;
    std::vector<double> work(n);
    for (int q = 0; q < n; ++q) {
        ProblemLayout L;
        std::string err;
        if (!build_problem_layout(descs[q], L, err)) {
            batch_free(b);
            return set_error("psba_batch_create: problem " + std::to_string(q) + ": " + err), PSBA_ERR_ARG;
        }
        rebase_problem(L.bp, (long long)dA.size(), (long long)iA.size(), r_total);
        dA.insert(dA.end(), L.dA.begin(), L.dA.end());
        iA.insert(iA.end(), L.iA.begin(), L.iA.end());
        r_total += L.nr;
        h.probs[q] = L.bp;
        work[q] = L.work;
    }
    // longest-first processing order (by observations, then reduced size)
    h.order.resize(n);
    for (int q = 0; q < n; ++q) h.order[q] = q;
    std::stable_sort(h.order.begin(), h.order.end(), [&](int a, int c) { return work[a] > work[c]; });
    h.nd = (long long)dA.size();
    h.ni = (long long)iA.size();
    h.nr = r_total;
    cudaError_t e = cudaStreamCreateWithFlags(&h.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&h.ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&h.ev1);
    if (e == cudaSuccess) e = cudaMalloc(&h.d_probs, sizeof(BatchProblem) * n);
    if (e == cudaSuccess) e = cudaMalloc(&h.d_order, sizeof(int) * n);
    if (e == cudaSuccess) e = cudaMalloc(&h.d_queue, sizeof(int));
    if (e == cudaSuccess) e = cudaMalloc(&h.d_res, sizeof(BatchResult) * n);
    if (e == cudaSuccess) e = cudaMalloc(&h.d_opts, sizeof(BatchOpts));
    if (e == cudaSuccess) e = cudaMalloc(&h.d_arena, sizeof(double) * std::max<long long>(h.nd, 1));
    if (e == cudaSuccess) e = cudaMalloc(&h.i_arena, sizeof(int) * std::max<long long>(h.ni, 1));
    if (e == cudaSuccess) e = cudaMalloc(&h.r_arena, sizeof(double) * std::max<long long>(h.nr, 1));
    if (e != cudaSuccess) {
        const int r = cuda_fail(e, "psba_batch_create");
        batch_free(b);
        return r;
    }
    h.bytes = sizeof(BatchProblem) * n + sizeof(double) * (h.nd + h.nr) + sizeof(int) * h.ni;
    e = cudaMemcpyAsync(h.d_probs, h.probs.data(), sizeof(BatchProblem) * n, cudaMemcpyHostToDevice, h.stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.d_order, h.order.data(), sizeof(int) * n, cudaMemcpyHostToDevice, h.stream);
    if (e == cudaSuccess && h.nd) e = cudaMemcpyAsync(h.d_arena, dA.data(), sizeof(double) * h.nd, cudaMemcpyHostToDevice, h.stream);
    if (e == cudaSuccess && h.ni) e = cudaMemcpyAsync(h.i_arena, iA.data(), sizeof(int) * h.ni, cudaMemcpyHostToDevice, h.stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h.stream);
    if (e != cudaSuccess) {
        const int r = cuda_fail(e, "psba_batch_create upload");
        batch_free(b);
        return r;
    }
    *out = b;
    return PSBA_OK;
}

int psba_batch_destroy(psba_batch *b)
{
    batch_free(b);
    return PSBA_OK;
}

int psba_batch_set_threads(psba_batch *b, int threads)
{
    if (!b || (threads != 128 && threads != 256 && threads != 512))
        return set_error("psba_batch_set_threads: 128, 256 or 512"), PSBA_ERR_ARG;
    b->hb.threads = threads;
    return PSBA_OK;
}

int psba_batch_reset_params(psba_batch *b)
{
    if (!b) return set_error("null batch"), PSBA_ERR_ARG;
    HostBatch &h = b->hb;
    for (int q = 0; q < h.n; ++q) {
        const BatchProblem &p = h.probs[q];
        cudaMemcpyAsync(h.d_arena + p.d_cams, h.d_arena + p.d_cams0, sizeof(double) * 6 * p.nc,
                        cudaMemcpyDeviceToDevice, h.stream);
        if (p.np)
            cudaMemcpyAsync(h.d_arena + p.d_pts, h.d_arena + p.d_pts0, sizeof(double) * 3 * p.np,
                            cudaMemcpyDeviceToDevice, h.stream);
    }
    const cudaError_t e = cudaStreamSynchronize(h.stream);
    return e == cudaSuccess ? PSBA_OK : cuda_fail(e, "psba_batch_reset_params");
}

int psba_batch_levmar(psba_batch *b, const psba_opts *opts, psba_batch_result *results, double *device_ms)
{
    if (!b || !opts) return set_error("null argument"), PSBA_ERR_ARG;
    if (opts->refine != 0) return set_error("psba_batch_levmar: refine is for the per-handle solver"), PSBA_ERR_ARG;
    HostBatch &h = b->hb;
    BatchOpts o;
    o.tau = opts->tau;
    o.stop_thresh = opts->stop_thresh;
    o.eps = opts->eps;
    o.max_iter = opts->max_iter;
    o.allow_switch = opts->allow_switch;
    o.precision = opts->precision;
    o.pad = 0;
    int sms = 0, dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const int key = opts->precision * 1024 + h.threads;
    static_assert(sizeof(BatchOpts) % 8 == 0, "BatchOpts");
    // The launch (queue reset + one persistent kernel) is captured into a CUDA
    // graph once per (precision, block size) and replayed; options travel in a
    // device copy so that the graph does not depend on them.
    cudaError_t e = cudaSuccess;
    if (h.graph == nullptr || h.graph_key != key) {
        if (h.graph) cudaGraphExecDestroy(h.graph);
        h.graph = nullptr;
        cudaGraph_t g = nullptr;
        e = cudaStreamBeginCapture(h.stream, cudaStreamCaptureModeThreadLocal);
        if (e != cudaSuccess) return cuda_fail(e, "psba_batch_levmar capture");
        cudaMemsetAsync(h.d_queue, 0, sizeof(int), h.stream);
        cudaMemsetAsync(h.d_res, 0, sizeof(BatchResult) * h.n, h.stream);  // every problem starts afresh
        const int grid = std::min(h.n, batch_blocks_per_sm(opts->precision, h.threads) * sms);
        launch_batch_lm(opts->precision, grid, h.threads, h.stream, h.d_probs, h.d_order, h.n, h.d_queue,
                        h.d_arena, h.i_arena, h.r_arena, h.d_opts, h.d_res);
        e = cudaStreamEndCapture(h.stream, &g);
        if (e == cudaSuccess) e = cudaGraphInstantiate(&h.graph, g, 0);
        if (g) cudaGraphDestroy(g);
        if (e != cudaSuccess) return cuda_fail(e, "psba_batch_levmar graph");
        h.graph_key = key;
    }
    e = cudaMemcpyAsync(h.d_opts, &o, sizeof(BatchOpts), cudaMemcpyHostToDevice, h.stream);
    if (e != cudaSuccess) return cuda_fail(e, "psba_batch_levmar options");
    cudaEventRecord(h.ev0, h.stream);
    e = cudaGraphLaunch(h.graph, h.stream);
    note_launch(1);  // the graph's one kernel
    cudaEventRecord(h.ev1, h.stream);
    if (e == cudaSuccess) e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaEventSynchronize(h.ev1);
    if (e != cudaSuccess) return cuda_fail(e, "psba_batch_levmar");
    float ms = 0.f;
    cudaEventElapsedTime(&ms, h.ev0, h.ev1);
    if (device_ms) *device_ms = ms;
    if (results) {
        std::vector<BatchResult> r(h.n);
        e = cudaMemcpy(r.data(), h.d_res, sizeof(BatchResult) * h.n, cudaMemcpyDeviceToHost);
        if (e != cudaSuccess) return cuda_fail(e, "psba_batch_levmar results");
        for (int q = 0; q < h.n; ++q) {
            results[q].status = r[q].status;
            results[q].iterations = r[q].iterations;
            results[q].n_trials = r[q].trials;
            results[q].n_linearizations = r[q].linearizations;
            results[q].initial_cost = r[q].initial_cost;
            results[q].final_cost = r[q].final_cost;
            results[q].mu = r[q].mu;
            results[q].p_L2 = r[q].p_L2;
            results[q].nu = r[q].nu;
            results[q].pad = 0;
        }
    }
    return PSBA_OK;
}

int psba_batch_get_params(psba_batch *b, int q, double *cams, double *pts)
{
    if (!b || q < 0 || q >= b->hb.n || !cams) return set_error("psba_batch_get_params: bad arguments"), PSBA_ERR_ARG;
    HostBatch &h = b->hb;
    const BatchProblem &p = h.probs[q];
    cudaError_t e = cudaMemcpy(cams, h.d_arena + p.d_cams, sizeof(double) * 6 * p.nc, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && p.np && pts)
        e = cudaMemcpy(pts, h.d_arena + p.d_pts, sizeof(double) * 3 * p.np, cudaMemcpyDeviceToHost);
    return e == cudaSuccess ? PSBA_OK : cuda_fail(e, "psba_batch_get_params");
}

size_t psba_batch_device_bytes(psba_batch *b) { return b ? b->hb.bytes : 0; }

int psba_batch_set_lanes_per_pair(psba_batch *b, const int *lanes)
{
    if (!b || !lanes) return set_error("null argument"), PSBA_ERR_ARG;
    HostBatch &h = b->hb;
    for (int q = 0; q < h.n; ++q) {
        const int l = lanes[q];
        if (l != 8 && l != 16 && l != 32) return set_error("lanes per pair must be 8, 16 or 32"), PSBA_ERR_ARG;
        h.probs[q].flags = (h.probs[q].flags & ~0xff) | l;
    }
    const cudaError_t e = cudaMemcpy(h.d_probs, h.probs.data(), sizeof(BatchProblem) * h.n, cudaMemcpyHostToDevice);
    return e == cudaSuccess ? PSBA_OK : cuda_fail(e, "psba_batch_set_lanes_per_pair");
}

}  // extern "C"

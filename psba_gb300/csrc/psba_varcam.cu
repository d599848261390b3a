// Camera-block stages for variable intrinsics: cnp = 11 (pose + fx, cx, cy,
// aspect, skew) and cnp = 16 (+ distortion k1, k2, p1, p2, k3).
//
// The reference fixes cnp = 6 in every kernel (CL_files/PSBA.cl:5); these
// are the same stages with cnp-wide camera blocks: A is 2 x cnp, W and Y are
// cnp x 3, U and the Schur blocks cnp x cnp.  The camera model
//   x = Xc/Zc, y = Yc/Zc, r2 = x^2 + y^2,
//   radial = 1 + k1 r2 + k2 r2^2 + k3 r2^3,
//   xd = radial x + 2 p1 x y + p2 (r2 + 2 x^2),
//   yd = radial y + p1 (r2 + 2 y^2) + 2 p2 x y,
//   u = fx xd + skew yd + cx,   v = fx aspect yd + cy
// is Bouguet's, in the order of the sba camera files (data/54camsvarKD.txt);
// without distortion it is the reference's pinhole.  The Jacobian is the
// chain rule through the camera table (rotation, its derivative, intrinsics
// and distortion, k_cam_tables).
//
// Work units are those of the 6-parameter kernels (camera chunks, camera-pair
// chunks); each unit is one CTA that stages its rows in shared memory and
// sums every block entry in a fixed order, so results are repeatable.  The
// mixed form stores A, W, Y in FP32 and sums FP32 products FLUSH at a time
// into FP64, like the 6-parameter kernels; the gradient is FP64 from exact
// products in both forms.
#include "psba_internal.h"

namespace psba {

namespace {

inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

constexpr int VC_THREADS = 128;
constexpr int VFLUSH = 8;

template <int CNP> __host__ __device__ constexpr int cam_nv() { return CNP * (CNP + 1) / 2 + CNP; }  // U upper + ga
template <int CNP> __host__ __device__ constexpr int diag_nv() { return CNP * (CNP + 1) / 2 + CNP; } // S lower + ea

// (r, c) of the v-th entry of the upper triangle, row-major
__host__ __device__ inline void upper_rc(int v, int n, int &r, int &c)
{
    r = 0;
    while (v >= n - r) {
        v -= n - r;
        ++r;
    }
    c = r + v;
}

// (r, c) of the v-th entry of the lower triangle, row-major
__host__ __device__ inline void lower_rc(int v, int &r, int &c)
{
    r = 0;
    while (v > r) {
        v -= r + 1;
        ++r;
    }
    c = v;
}

}  // namespace

// ---------------------------------------------------------------------------
// Linearization: one thread per observation.  Projection and residual in
// FP64; derivatives evaluated in R from the FP64 quantities.
template <typename R, int CNP>
__global__ void __launch_bounds__(256) k_linearize_v(int no, const int *__restrict__ obs_pt,
                                                     const int *__restrict__ obs_cam,
                                                     const double *__restrict__ meas,
                                                     const double *__restrict__ pts,
                                                     const double *__restrict__ tab, double coeff,
                                                     const double *__restrict__ wt,
                                                     R *__restrict__ ex, R *__restrict__ A,
                                                     R *__restrict__ B, R *__restrict__ W)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= no) return;
    const int i = obs_pt[o], j = obs_cam[o];
    const CamTab *T = reinterpret_cast<const CamTab *>(tab + (size_t)CAMTAB * j);
    const double X0 = pts[3 * i], X1 = pts[3 * i + 1], X2 = pts[3 * i + 2];
    const double xc = T->M[0] * X0 + T->M[1] * X1 + T->M[2] * X2 + T->t[0];
    const double yc = T->M[3] * X0 + T->M[4] * X1 + T->M[5] * X2 + T->t[1];
    const double zc = T->M[6] * X0 + T->M[7] * X1 + T->M[8] * X2 + T->t[2];
    const double iz = 1.0 / zc;
    double u, v, xd, yd, x = xc * iz, y = yc * iz;
    double Dd00 = 1.0, Dd01 = 0.0, Dd10 = 0.0, Dd11 = 1.0, r2 = x * x + y * y;
    if (CNP == 16) {
        const double *kc = T->kc;
        const double radial = 1.0 + r2 * (kc[0] + r2 * (kc[1] + r2 * kc[4]));
        xd = radial * x + 2.0 * kc[2] * x * y + kc[3] * (r2 + 2.0 * x * x);
        yd = radial * y + kc[2] * (r2 + 2.0 * y * y) + 2.0 * kc[3] * x * y;
        u = T->fx * xd + T->sk * yd + T->cx;
        v = T->fy * yd + T->cy;
        const double dr = kc[0] + r2 * (2.0 * kc[1] + 3.0 * kc[4] * r2);
        Dd00 = radial + 2.0 * x * x * dr + 2.0 * kc[2] * y + 6.0 * kc[3] * x;
        Dd01 = 2.0 * x * y * dr + 2.0 * kc[2] * x + 2.0 * kc[3] * y;
        Dd10 = Dd01;
        Dd11 = radial + 2.0 * y * y * dr + 6.0 * kc[2] * y + 2.0 * kc[3] * x;
    } else {
        u = (T->fx * xc + T->sk * yc + T->cx * zc) * iz;
        v = (T->fy * yc + T->cy * zc) * iz;
        xd = x;
        yd = y;
    }
    double e0 = meas[2 * (size_t)o] - u, e1 = meas[2 * (size_t)o + 1] - v, wa = 1.0, wb = 0.0, wc = 1.0;
    if (wt) {  // whitening: e <- L e, J rows <- L J
        wa = wt[3 * (size_t)o];
        wb = wt[3 * (size_t)o + 1];
        wc = wt[3 * (size_t)o + 2];
        const double t0 = wa * e0 + wb * e1;
        e1 = wc * e1;
        e0 = t0;
    }
    ex[2 * (size_t)o] = (R)e0;
    ex[2 * (size_t)o + 1] = (R)e1;
    // H = d(u,v)/dXc = P Dd N
    const R fx = (R)T->fx, sk = (R)T->sk, fy = (R)T->fy, izr = (R)iz, xr = (R)x, yr = (R)y;
    const R pd00 = fx * (R)Dd00 + sk * (R)Dd10, pd01 = fx * (R)Dd01 + sk * (R)Dd11;
    const R pd10 = fy * (R)Dd10, pd11 = fy * (R)Dd11;
    R H[2][3];
    H[0][0] = pd00 * izr;
    H[0][1] = pd01 * izr;
    H[0][2] = -(pd00 * xr + pd01 * yr) * izr;
    H[1][0] = pd10 * izr;
    H[1][1] = pd11 * izr;
    H[1][2] = -(pd10 * xr + pd11 * yr) * izr;
    R a[2][CNP], b[2][3];
    const R Xr0 = (R)X0, Xr1 = (R)X1, Xr2 = (R)X2;
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        const double *Dm = T->D + 9 * m;
        const R g0 = (R)Dm[0] * Xr0 + (R)Dm[1] * Xr1 + (R)Dm[2] * Xr2;
        const R g1 = (R)Dm[3] * Xr0 + (R)Dm[4] * Xr1 + (R)Dm[5] * Xr2;
        const R g2 = (R)Dm[6] * Xr0 + (R)Dm[7] * Xr1 + (R)Dm[8] * Xr2;
#pragma unroll
        for (int r = 0; r < 2; ++r) {
            a[r][m] = H[r][0] * g0 + H[r][1] * g1 + H[r][2] * g2;
            a[r][3 + m] = H[r][m];
            b[r][m] = H[r][0] * (R)T->M[m] + H[r][1] * (R)T->M[3 + m] + H[r][2] * (R)T->M[6 + m];
        }
    }
    const R xdr = (R)xd, ydr = (R)yd;
    a[0][6] = xdr;          a[1][6] = (R)T->ar * ydr;
    a[0][7] = (R)1;         a[1][7] = (R)0;
    a[0][8] = (R)0;         a[1][8] = (R)1;
    a[0][9] = (R)0;         a[1][9] = fx * ydr;
    a[0][10] = ydr;         a[1][10] = (R)0;
    if constexpr (CNP == 16) {
        const R r2r = (R)r2, r4 = r2r * r2r, r6 = r4 * r2r;
        const R dxd[5] = {xr * r2r, xr * r4, (R)2 * xr * yr, r2r + (R)2 * xr * xr, xr * r6};
        const R dyd[5] = {yr * r2r, yr * r4, r2r + (R)2 * yr * yr, (R)2 * xr * yr, yr * r6};
#pragma unroll
        for (int k = 0; k < 5; ++k) {
            a[0][11 + k] = fx * dxd[k] + sk * dyd[k];
            a[1][11 + k] = fy * dyd[k];
        }
    }
    if (wt) {
        const R ra = (R)wa, rb = (R)wb, rc = (R)wc;
#pragma unroll
        for (int c = 0; c < CNP; ++c) {
            const R a0 = a[0][c], a1 = a[1][c];
            a[0][c] = ra * a0 + rb * a1;
            a[1][c] = rc * a1;
        }
#pragma unroll
        for (int c = 0; c < 3; ++c) {
            const R b0 = b[0][c], b1 = b[1][c];
            b[0][c] = ra * b0 + rb * b1;
            b[1][c] = rc * b1;
        }
    }
    R *Ao = A + 2 * CNP * (size_t)o, *Bo = B + 6 * (size_t)o, *Wo = W + 3 * CNP * (size_t)o;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
#pragma unroll
        for (int c = 0; c < CNP; ++c) Ao[r * CNP + c] = a[r][c];
#pragma unroll
        for (int c = 0; c < 3; ++c) Bo[r * 3 + c] = b[r][c];
    }
    const R cf = (R)coeff;
#pragma unroll
    for (int r = 0; r < CNP; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) Wo[r * 3 + c] = cf * (a[0][r] * b[0][c] + a[1][r] * b[1][c]);
}

// Cost of one observation with distortion (cnp 16); the 6- and 11-parameter
// models use k_residual's pinhole expression.
__global__ void __launch_bounds__(256) k_residual_dist(int no, const int *__restrict__ obs_pt,
                                                       const int *__restrict__ obs_cam,
                                                       const double *__restrict__ meas,
                                                       const double *__restrict__ pts,
                                                       const double *__restrict__ dpb,
                                                       const double *__restrict__ tab,
                                                       const double *__restrict__ wt,
                                                       double *__restrict__ ex_out,
                                                       double *__restrict__ partial)
{
    __shared__ double red[256 / 32];
    // the grid's threads over the observations o, o + grid, ... (the grid of
    // k_residual: a few blocks per SM), each thread's squares in its order
    double sq = 0.0;
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < no; o += gridDim.x * blockDim.x) {
        const int i = obs_pt[o], j = obs_cam[o];
        double X[3];
        for (int m = 0; m < 3; ++m) X[m] = dpb ? pts[3 * i + m] + dpb[3 * i + m] : pts[3 * i + m];
        const CamTab *T = reinterpret_cast<const CamTab *>(tab + (size_t)CAMTAB * j);
        const double xc = T->M[0] * X[0] + T->M[1] * X[1] + T->M[2] * X[2] + T->t[0];
        const double yc = T->M[3] * X[0] + T->M[4] * X[1] + T->M[5] * X[2] + T->t[1];
        const double zc = T->M[6] * X[0] + T->M[7] * X[1] + T->M[8] * X[2] + T->t[2];
        const double iz = 1.0 / zc, x = xc * iz, y = yc * iz;
        const double *kc = T->kc;
        const double r2 = x * x + y * y;
        const double radial = 1.0 + r2 * (kc[0] + r2 * (kc[1] + r2 * kc[4]));
        const double xd = radial * x + 2.0 * kc[2] * x * y + kc[3] * (r2 + 2.0 * x * x);
        const double yd = radial * y + kc[2] * (r2 + 2.0 * y * y) + 2.0 * kc[3] * x * y;
        double e0 = meas[2 * (size_t)o] - (T->fx * xd + T->sk * yd + T->cx);
        double e1 = meas[2 * (size_t)o + 1] - (T->fy * yd + T->cy);
        if (wt) {
            const double t0 = wt[3 * (size_t)o] * e0 + wt[3 * (size_t)o + 1] * e1;
            e1 = wt[3 * (size_t)o + 2] * e1;
            e0 = t0;
        }
        if (ex_out) {
            ex_out[2 * (size_t)o] = e0;
            ex_out[2 * (size_t)o + 1] = e1;
        }
        sq = fma(e0, e0, fma(e1, e1, sq));
    }
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = red[0];
        for (int w = 1; w < 256 / 32; ++w) a += red[w];
        partial[blockIdx.x] = a;
    }
}

// ---------------------------------------------------------------------------
// U_j (upper triangle) and ga_j per camera unit: the unit's A rows and
// residuals are staged in shared memory 32 observations at a time; thread t
// owns entries t, t + 128, ... and sums them over the unit in order.
template <typename R, int CNP>
__global__ void __launch_bounds__(VC_THREADS) k_camera_partial_v(const CamUnit *__restrict__ units,
                                                                 const int *__restrict__ cam_obs,
                                                                 const R *__restrict__ A,
                                                                 const R *__restrict__ ex,
                                                                 double *__restrict__ partial)
{
    constexpr int NV = cam_nv<CNP>(), NU = CNP * (CNP + 1) / 2, PER = (NV + VC_THREADS - 1) / VC_THREADS;
    constexpr int CH = 32;
    __shared__ R sa[CH][2 * CNP];
    __shared__ R se[CH][2];
    const CamUnit u = units[blockIdx.x];
    double acc[PER];
    int er[PER], ec[PER];
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        acc[q] = 0.0;
        const int v = threadIdx.x + q * VC_THREADS;
        er[q] = ec[q] = -1;
        if (v < NU) upper_rc(v, CNP, er[q], ec[q]);
        else if (v < NV) er[q] = v - NU;  // gradient row
    }
    for (int t0 = 0; t0 < u.count; t0 += CH) {
        const int n = min(CH, u.count - t0);
        __syncthreads();
        for (int e = threadIdx.x; e < n * 2 * CNP; e += VC_THREADS) {
            const int t = e / (2 * CNP), k = e % (2 * CNP);
            sa[t][k] = A[2 * CNP * (size_t)cam_obs[u.begin + t0 + t] + k];
        }
        for (int e = threadIdx.x; e < n * 2; e += VC_THREADS)
            se[e / 2][e % 2] = ex[2 * (size_t)cam_obs[u.begin + t0 + e / 2] + e % 2];
        __syncthreads();
#pragma unroll
        for (int q = 0; q < PER; ++q) {
            const int v = threadIdx.x + q * VC_THREADS;
            if (v >= NV) continue;
            const int r = er[q], c = ec[q];
            if (v < NU) {
                for (int f0 = 0; f0 < n; f0 += VFLUSH) {
                    R part = (R)0;
                    const int f1 = min(n, f0 + VFLUSH);
                    for (int t = f0; t < f1; ++t) part = part + sa[t][r] * sa[t][c] + sa[t][CNP + r] * sa[t][CNP + c];
                    acc[q] += (double)part;
                }
            } else {
                for (int t = 0; t < n; ++t)
                    acc[q] = acc[q] + (double)sa[t][r] * (double)se[t][0] + (double)sa[t][CNP + r] * (double)se[t][1];
            }
        }
    }
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int v = threadIdx.x + q * VC_THREADS;
        if (v < NV) partial[(size_t)blockIdx.x * NV + v] = acc[q];
    }
}

template <int CNP>
__global__ void k_camera_finish_v(int nc, const int *__restrict__ unit_start, const double *__restrict__ partial,
                                  double coeff, double *__restrict__ U, double *__restrict__ g,
                                  double *__restrict__ uvdiag)
{
    constexpr int NV = cam_nv<CNP>(), NU = CNP * (CNP + 1) / 2;
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nc * NV) return;
    const int j = id / NV, v = id % NV;
    double sum = 0.0;
    for (int u = unit_start[j]; u < unit_start[j + 1]; ++u) sum += partial[(size_t)u * NV + v];
    sum = coeff * sum;
    if (v >= NU) {
        g[CNP * (size_t)j + (v - NU)] = sum;
        return;
    }
    int r, c;
    upper_rc(v, CNP, r, c);
    U[(size_t)CNP * CNP * j + r * CNP + c] = sum;
    U[(size_t)CNP * CNP * j + c * CNP + r] = sum;
    if (r == c) uvdiag[CNP * (size_t)j + r] = sum;
}

// Y = W V^-1 per observation (V^-1 FP64, products FP64, stored in R).
template <typename R, int CNP>
__global__ void __launch_bounds__(256) k_yblocks_v(int no, const int *__restrict__ obs_pt, const R *__restrict__ W,
                                                   const double *__restrict__ Vinv, R *__restrict__ Y)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= no) return;
    const double *vi = Vinv + 6 * (size_t)obs_pt[o];
    const double s00 = vi[0], s01 = vi[1], s02 = vi[2], s11 = vi[3], s12 = vi[4], s22 = vi[5];
    const R *w = W + 3 * CNP * (size_t)o;
    R *y = Y + 3 * CNP * (size_t)o;
#pragma unroll 4
    for (int r = 0; r < CNP; ++r) {
        const double w0 = w[3 * r], w1 = w[3 * r + 1], w2 = w[3 * r + 2];
        y[3 * r] = (R)(w0 * s00 + w1 * s01 + w2 * s02);
        y[3 * r + 1] = (R)(w0 * s01 + w1 * s11 + w2 * s12);
        y[3 * r + 2] = (R)(w0 * s02 + w1 * s12 + w2 * s22);
    }
}

// Off-diagonal Schur blocks: one CTA per unit of <= SCHUR_CHUNK common
// points of a camera pair (k > l); the unit's Y_a and W_b rows are staged in
// shared memory; thread t owns entries t, t + 128, ... of the cnp x cnp block.
template <typename R, int CNP>
__global__ void __launch_bounds__(VC_THREADS) k_schur_off_v(const SchurUnit *__restrict__ units,
                                                            const int *__restrict__ pa, const int *__restrict__ pb,
                                                            const R *__restrict__ Y, const R *__restrict__ W,
                                                            double *__restrict__ partial)
{
    constexpr int NE = CNP * CNP, PER = (NE + VC_THREADS - 1) / VC_THREADS;
    __shared__ R sy[SCHUR_CHUNK][3 * CNP], sw[SCHUR_CHUNK][3 * CNP];
    const SchurUnit u = units[blockIdx.x];
    for (int e = threadIdx.x; e < u.count * 3 * CNP; e += VC_THREADS) {
        const int t = e / (3 * CNP), k = e % (3 * CNP);
        sy[t][k] = Y[3 * CNP * (size_t)pa[u.begin + t] + k];
        sw[t][k] = W[3 * CNP * (size_t)pb[u.begin + t] + k];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int v = threadIdx.x + q * VC_THREADS;
        if (v >= NE) continue;
        const int r = v / CNP, c = v % CNP;
        double acc = 0.0;
        if constexpr (sizeof(R) == 8) {
            for (int t = 0; t < u.count; ++t) {
                acc = fma((double)sy[t][3 * r], (double)sw[t][3 * c], acc);
                acc = fma((double)sy[t][3 * r + 1], (double)sw[t][3 * c + 1], acc);
                acc = fma((double)sy[t][3 * r + 2], (double)sw[t][3 * c + 2], acc);
            }
        } else {
            for (int f0 = 0; f0 < u.count; f0 += VFLUSH) {
                R part = (R)0;
                const int f1 = min(u.count, f0 + VFLUSH);
                for (int t = f0; t < f1; ++t) {
                    part = fma(sy[t][3 * r], sw[t][3 * c], part);
                    part = fma(sy[t][3 * r + 1], sw[t][3 * c + 1], part);
                    part = fma(sy[t][3 * r + 2], sw[t][3 * c + 2], part);
                }
                acc += (double)part;
            }
        }
        partial[(size_t)u.out * NE + v] = acc;
    }
}

// Diagonal Schur blocks and ea: one CTA per unit of <= DIAG_CHUNK
// observations of a camera; lower-triangle entries of sum Y W^T and the
// cnp sums of Y gb.
template <typename R, int CNP>
__global__ void __launch_bounds__(VC_THREADS) k_schur_diag_v(const SchurUnit *__restrict__ units,
                                                             const int *__restrict__ cam_obs,
                                                             const int *__restrict__ obs_pt,
                                                             const R *__restrict__ Y, const R *__restrict__ W,
                                                             const double *__restrict__ gb,
                                                             double *__restrict__ partial)
{
    constexpr int NV = diag_nv<CNP>(), NL = CNP * (CNP + 1) / 2, PER = (NV + VC_THREADS - 1) / VC_THREADS;
    __shared__ R sy[DIAG_CHUNK][3 * CNP], sw[DIAG_CHUNK][3 * CNP];
    __shared__ double sg[DIAG_CHUNK][3];
    const SchurUnit u = units[blockIdx.x];
    for (int e = threadIdx.x; e < u.count * 3 * CNP; e += VC_THREADS) {
        const int t = e / (3 * CNP), k = e % (3 * CNP);
        const int o = cam_obs[u.begin + t];
        sy[t][k] = Y[3 * CNP * (size_t)o + k];
        sw[t][k] = W[3 * CNP * (size_t)o + k];
    }
    for (int e = threadIdx.x; e < u.count * 3; e += VC_THREADS) {
        const int t = e / 3, k = e % 3;
        sg[t][k] = gb[3 * (size_t)obs_pt[cam_obs[u.begin + t]] + k];
    }
    __syncthreads();
#pragma unroll
    for (int q = 0; q < PER; ++q) {
        const int v = threadIdx.x + q * VC_THREADS;
        if (v >= NV) continue;
        double acc = 0.0;
        if (v < NL) {
            int r, c;
            lower_rc(v, r, c);
            for (int f0 = 0; f0 < u.count; f0 += VFLUSH) {
                R part = (R)0;
                const int f1 = min(u.count, f0 + VFLUSH);
                for (int t = f0; t < f1; ++t) {
                    part = fma(sy[t][3 * r], sw[t][3 * c], part);
                    part = fma(sy[t][3 * r + 1], sw[t][3 * c + 1], part);
                    part = fma(sy[t][3 * r + 2], sw[t][3 * c + 2], part);
                }
                acc += (double)part;
            }
        } else {
            // ea sums: FP64 from the exact products in both forms (ea cancels
            // near the optimum)
            const int r = v - NL;
            for (int t = 0; t < u.count; ++t) {
                acc = fma((double)sy[t][3 * r], sg[t][0], acc);
                acc = fma((double)sy[t][3 * r + 1], sg[t][1], acc);
                acc = fma((double)sy[t][3 * r + 2], sg[t][2], acc);
            }
        }
        partial[(size_t)u.out * NV + v] = acc;
    }
}

template <int CNP>
__global__ void k_schur_reduce_v(int n_pairs, int nc, int Np, const int *__restrict__ pair_kl,
                                 const int *__restrict__ off_start, const double *__restrict__ off_partial,
                                 const int *__restrict__ diag_start, const double *__restrict__ diag_partial,
                                 const double *__restrict__ U, const double *__restrict__ g, double mu,
                                 double *__restrict__ S, double *__restrict__ rhs)
{
    constexpr int NE = CNP * CNP, NV = diag_nv<CNP>(), NL = CNP * (CNP + 1) / 2;
    const long long id = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long n_off = (long long)n_pairs * NE;
    if (id < n_off) {
        const int p = (int)(id / NE), v = (int)(id % NE);
        double sum = 0.0;
        for (int u = off_start[p]; u < off_start[p + 1]; ++u) sum += off_partial[(size_t)u * NE + v];
        const int k = pair_kl[2 * p], l = pair_kl[2 * p + 1];
        S[(size_t)(CNP * k + v / CNP) * Np + CNP * l + v % CNP] = -sum;
        return;
    }
    const long long id2 = id - n_off;
    if (id2 >= (long long)nc * NV) return;
    const int k = (int)(id2 / NV), v = (int)(id2 % NV);
    double sum = 0.0;
    for (int u = diag_start[k]; u < diag_start[k + 1]; ++u) sum += diag_partial[(size_t)u * NV + v];
    if (v >= NL) {
        const int r = v - NL;
        rhs[CNP * k + r] = g[CNP * k + r] - sum;
        return;
    }
    int r, c;
    lower_rc(v, r, c);
    const double uu = U[(size_t)CNP * CNP * k + r * CNP + c];
    S[(size_t)(CNP * k + r) * Np + CNP * k + c] = (r == c ? uu + mu : uu) - sum;
}

// eb = gb - sum_j W_ij^T dpa_j, dpb = V^-1 eb, gain-ratio partials (as k_eb_dpb).
template <typename R, int CNP>
__global__ void __launch_bounds__(256) k_eb_dpb_v(int np, int ncp, const int *__restrict__ pt_start,
                                                  const int *__restrict__ pt_order,
                                                  const int *__restrict__ obs_cam, const R *__restrict__ W,
                                                  const double *__restrict__ Vinv, const double *__restrict__ g,
                                                  double mu, double *__restrict__ dp, double *__restrict__ eb,
                                                  double *__restrict__ partial)
{
    __shared__ double r0[256], r1[256];
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    double s_sq = 0.0, s_rho = 0.0;
    if (t < np) {
        const int i = pt_order[t];
        double e0 = 0, e1 = 0, e2 = 0;
        for (int o = pt_start[i]; o < pt_start[i + 1]; ++o) {
            const R *w = W + 3 * CNP * (size_t)o;
            const double *da = dp + CNP * (size_t)obs_cam[o];
#pragma unroll 4
            for (int k = 0; k < CNP; ++k) {
                const double dk = da[k];
                e0 = e0 + (double)w[3 * k] * dk;
                e1 = e1 + (double)w[3 * k + 1] * dk;
                e2 = e2 + (double)w[3 * k + 2] * dk;
            }
        }
        const double *gb = g + ncp + 3 * (size_t)i;
        e0 = gb[0] - e0;
        e1 = gb[1] - e1;
        e2 = gb[2] - e2;
        eb[3 * (size_t)i] = e0;
        eb[3 * (size_t)i + 1] = e1;
        eb[3 * (size_t)i + 2] = e2;
        const double *vi = Vinv + 6 * (size_t)i;
        const double d0 = vi[0] * e0 + vi[1] * e1 + vi[2] * e2;
        const double d1 = vi[1] * e0 + vi[3] * e1 + vi[4] * e2;
        const double d2 = vi[2] * e0 + vi[4] * e1 + vi[5] * e2;
        double *db = dp + ncp + 3 * (size_t)i;
        db[0] = d0;
        db[1] = d1;
        db[2] = d2;
        s_sq = d0 * d0 + d1 * d1 + d2 * d2;
        s_rho = d0 * (mu * d0 + gb[0]) + d1 * (mu * d1 + gb[1]) + d2 * (mu * d2 + gb[2]);
    }
    r0[threadIdx.x] = s_sq;
    r1[threadIdx.x] = s_rho;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            r0[threadIdx.x] += r0[threadIdx.x + st];
            r1[threadIdx.x] += r1[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partial[2 * blockIdx.x] = r0[0];
        partial[2 * blockIdx.x + 1] = r1[0];
    }
}

template <typename R, int CNP>
__global__ void k_jmultiply_v(int no, int ncp, const int *__restrict__ obs_pt, const int *__restrict__ obs_cam,
                              const R *__restrict__ A, const R *__restrict__ B, const double *__restrict__ x,
                              double *__restrict__ out)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= no) return;
    const double *xa = x + CNP * (size_t)obs_cam[o];
    const double *xb = x + ncp + 3 * (size_t)obs_pt[o];
    const R *a = A + 2 * CNP * (size_t)o;
    const R *b = B + 6 * (size_t)o;
    for (int k = 0; k < 2; ++k) {
        double s = 0.0;
        for (int m = 0; m < CNP; ++m) s += (double)a[CNP * k + m] * xa[m];
        for (int m = 0; m < 3; ++m) s += (double)b[3 * k + m] * xb[m];
        out[2 * (size_t)o + k] = s;
    }
}

// ---------------------------------------------------------------- launchers

namespace {

template <typename R, int CNP>
void linearize_t(const DeviceProblem &d, double coeff, cudaStream_t s)
{
    k_linearize_v<R, CNP><<<ceil_div(d.no, 256), 256, 0, s>>>(d.no, d.obs_pt, d.obs_cam, d.meas, d.pts, d.camtab,
                                                              coeff, d.wt, (R *)d.ex, (R *)d.A, (R *)d.B, (R *)d.W);
}

template <typename R, int CNP>
void camera_t(const DeviceProblem &d, double coeff, cudaStream_t s)
{
    if (d.n_cam_units > 0) {
        k_camera_partial_v<R, CNP><<<d.n_cam_units, VC_THREADS, 0, s>>>(d.cam_units, d.cam_obs, (const R *)d.A,
                                                                        (const R *)d.ex, d.cam_partial);
        note_launch(1);
    }
    k_camera_finish_v<CNP><<<ceil_div((long long)d.nc * cam_nv<CNP>(), 128), 128, 0, s>>>(
        d.nc, d.cam_unit_start, d.cam_partial, coeff, d.U, d.g, d.uvdiag);
    note_launch(1);
}

template <typename R, int CNP>
void schur_off_t(const DeviceProblem &d, cudaStream_t s)
{
    if (d.n_off_units == 0) return;
    k_schur_off_v<R, CNP><<<d.n_off_units, VC_THREADS, 0, s>>>(d.off_units, d.pair_a, d.pair_b, (const R *)d.Y,
                                                               (const R *)d.W, d.schur_partial);
    note_launch(1);
}

template <typename R, int CNP>
void schur_diag_t(const DeviceProblem &d, cudaStream_t s)
{
    if (d.n_diag_units == 0) return;
    double *diag_partial = d.schur_partial + (size_t)d.n_off_units * CNP * CNP;
    k_schur_diag_v<R, CNP><<<d.n_diag_units, VC_THREADS, 0, s>>>(d.diag_units, d.cam_obs, d.obs_pt, (const R *)d.Y,
                                                                 (const R *)d.W, d.g + d.N, diag_partial);
    note_launch(1);
}

template <int CNP>
void reduce_t(const DeviceProblem &d, double mu, cudaStream_t s)
{
    double *off_partial = d.schur_partial;
    double *diag_partial = d.schur_partial + (size_t)d.n_off_units * CNP * CNP;
    const long long total = (long long)d.n_pairs * CNP * CNP + (long long)d.nc * diag_nv<CNP>();
    k_schur_reduce_v<CNP><<<ceil_div(total, 128), 128, 0, s>>>(d.n_pairs, d.nc, d.Np, d.pair_kl, d.off_unit_start,
                                                               off_partial, d.diag_unit_start, diag_partial, d.U,
                                                               d.g, mu, d.S, d.rhs);
    note_launch(1);
}

}  // namespace

size_t varcam_cam_partial(int cnp) { return cnp == 11 ? cam_nv<11>() : cam_nv<16>(); }
size_t varcam_diag_partial(int cnp) { return cnp == 11 ? diag_nv<11>() : diag_nv<16>(); }

#define VC_DISPATCH(F, ...)                                                      \
    do {                                                                         \
        const bool f64 = d.prec == PSBA_PREC_FP64;                               \
        if (d.cnp == 11) {                                                       \
            if (f64) F<double, 11>(__VA_ARGS__); else F<float, 11>(__VA_ARGS__); \
        } else {                                                                 \
            if (f64) F<double, 16>(__VA_ARGS__); else F<float, 16>(__VA_ARGS__); \
        }                                                                        \
    } while (0)

void launch_linearize_v(const DeviceProblem &d, double coeff, cudaStream_t s)
{
    if (d.no == 0) return;
    VC_DISPATCH(linearize_t, d, coeff, s);
    note_launch(1);
}

void launch_camera_blocks_v(const DeviceProblem &d, double coeff, cudaStream_t s)
{
    VC_DISPATCH(camera_t, d, coeff, s);
}

void launch_yblocks_v(const DeviceProblem &d, cudaStream_t s)
{
    if (d.no == 0) return;
    const bool f64 = d.prec == PSBA_PREC_FP64;
    const int nb = ceil_div(d.no, 256);
    if (d.cnp == 11) {
        if (f64) k_yblocks_v<double, 11><<<nb, 256, 0, s>>>(d.no, d.obs_pt, d.W, d.Vinv, d.Y);
        else k_yblocks_v<float, 11><<<nb, 256, 0, s>>>(d.no, d.obs_pt, (const float *)d.W, d.Vinv, (float *)d.Y);
    } else {
        if (f64) k_yblocks_v<double, 16><<<nb, 256, 0, s>>>(d.no, d.obs_pt, d.W, d.Vinv, d.Y);
        else k_yblocks_v<float, 16><<<nb, 256, 0, s>>>(d.no, d.obs_pt, (const float *)d.W, d.Vinv, (float *)d.Y);
    }
    note_launch(1);
}

void launch_schur_off_v(const DeviceProblem &d, cudaStream_t s) { VC_DISPATCH(schur_off_t, d, s); }

void launch_schur_diag_v(const DeviceProblem &d, cudaStream_t s) { VC_DISPATCH(schur_diag_t, d, s); }

void launch_schur_reduce_v(const DeviceProblem &d, double mu, cudaStream_t s)
{
    if (d.cnp == 11) reduce_t<11>(d, mu, s);
    else reduce_t<16>(d, mu, s);
}

void launch_eb_dpb_v(const DeviceProblem &d, double mu, int nblocks, cudaStream_t s)
{
    const bool f64 = d.prec == PSBA_PREC_FP64;
    if (d.cnp == 11) {
        if (f64) k_eb_dpb_v<double, 11><<<nblocks, 256, 0, s>>>(d.np, d.N, d.pt_start, d.pt_order, d.obs_cam, d.W, d.Vinv, d.g, mu, d.dp, d.eb, d.red_partial);
        else k_eb_dpb_v<float, 11><<<nblocks, 256, 0, s>>>(d.np, d.N, d.pt_start, d.pt_order, d.obs_cam, (const float *)d.W, d.Vinv, d.g, mu, d.dp, d.eb, d.red_partial);
    } else {
        if (f64) k_eb_dpb_v<double, 16><<<nblocks, 256, 0, s>>>(d.np, d.N, d.pt_start, d.pt_order, d.obs_cam, d.W, d.Vinv, d.g, mu, d.dp, d.eb, d.red_partial);
        else k_eb_dpb_v<float, 16><<<nblocks, 256, 0, s>>>(d.np, d.N, d.pt_start, d.pt_order, d.obs_cam, (const float *)d.W, d.Vinv, d.g, mu, d.dp, d.eb, d.red_partial);
    }
    note_launch(1);
}

void launch_jmultiply_v(const DeviceProblem &d, const double *x, double *out, cudaStream_t s)
{
    if (d.no == 0) return;
    const bool f64 = d.prec == PSBA_PREC_FP64;
    const int nb = ceil_div(d.no, 256);
    if (d.cnp == 11) {
        if (f64) k_jmultiply_v<double, 11><<<nb, 256, 0, s>>>(d.no, d.N, d.obs_pt, d.obs_cam, d.A, d.B, x, out);
        else k_jmultiply_v<float, 11><<<nb, 256, 0, s>>>(d.no, d.N, d.obs_pt, d.obs_cam, (const float *)d.A, (const float *)d.B, x, out);
    } else {
        if (f64) k_jmultiply_v<double, 16><<<nb, 256, 0, s>>>(d.no, d.N, d.obs_pt, d.obs_cam, d.A, d.B, x, out);
        else k_jmultiply_v<float, 16><<<nb, 256, 0, s>>>(d.no, d.N, d.obs_pt, d.obs_cam, (const float *)d.A, (const float *)d.B, x, out);
    }
    note_launch(1);
}

void launch_residual_dist(const DeviceProblem &d, const double *tab, const double *pts, const double *dpb,
                          double *ex_out, double *partial, int nblocks, cudaStream_t s)
{
    k_residual_dist<<<nblocks, 256, 0, s>>>(d.no, d.obs_pt, d.obs_cam, d.meas, pts, dpb, tab, d.wt, ex_out, partial);
    note_launch(1);
}

}  // namespace psba

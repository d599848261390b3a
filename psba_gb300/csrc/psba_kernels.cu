// Sparse stages of one Levenberg-Marquardt / dogleg iteration, FP64, sm_103a.
//
// Layout in HBM (all per-observation arrays follow the observation order,
// which is (point, camera) sorted as the reference's generate_idxs,
// PSBA/misc.cpp:189-197):
//   ex 2, A 12 (2x6 row-major), B 6 (2x3), W 18 (6x3), Y 18 (6x3) doubles per
//   observation; V and V^-1 6 doubles per point (upper triangle 00 01 02 11 12
//   22); U 36 per camera; g = [ga (6C) | gb (3P)].
// Every reduction runs in a fixed order (no floating-point atomics), so a
// solve is bit-for-bit repeatable.
#include <mutex>

#include "psba_internal.h"

namespace psba {

static inline int ceil_div(long long a, long long b) { return (int)((a + b - 1) / b); }

// Per-observation arrays are stored in R = double (PSBA_PREC_FP64) or
// R = float (PSBA_PREC_MIXED).  Every per-observation array has an even
// number of entries, so pairs are loaded and stored as double2 / float2.
template <typename R> struct Pair;
template <> struct Pair<double> { using T = double2; };
template <> struct Pair<float> { using T = float2; };

template <typename R>
__device__ __forceinline__ void st2(R *p, R a, R b)
{
    typename Pair<R>::T v;
    v.x = a;
    v.y = b;
    *reinterpret_cast<typename Pair<R>::T *>(p) = v;
}

template <typename R>
__device__ __forceinline__ void ld2(const R *p, R &a, R &b)
{
    const typename Pair<R>::T v = __ldg(reinterpret_cast<const typename Pair<R>::T *>(p));
    a = v.x;
    b = v.y;
}

template <typename R, int N>
__device__ __forceinline__ void ldn(const R *p, R *out)
{
#pragma unroll
    for (int e = 0; e < N / 2; ++e) ld2(p + 2 * e, out[2 * e], out[2 * e + 1]);
}

template <typename R, int N>
__device__ __forceinline__ void stn(R *p, const R *in)
{
#pragma unroll
    for (int e = 0; e < N / 2; ++e) st2(p + 2 * e, in[2 * e], in[2 * e + 1]);
}

template <typename R> __host__ __device__ constexpr bool is_fp64() { return sizeof(R) == 8; }

// Mixed precision: FP32 products summed in FP32 over FLUSH consecutive
// terms, then added into the FP64 accumulator.
constexpr int FLUSH = 8;

// ---------------------------------------------------------------------------
// The last block of a launch to finish (by a ticket in global memory) sums
// the launch's per-block partials into *dst in index order, so the result
// does not depend on which block that is, and resets the ticket for the next
// launch.  Thread 0 of every block calls it after writing the block's
// partial; blockDim.x == 256.
__device__ bool take_last_ticket(int *ticket)
{
    __shared__ int last;
    if (threadIdx.x == 0) {
        __threadfence();  // the block's partial before its ticket
        last = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
    }
    __syncthreads();
    if (last) __threadfence();
    return last;
}

__device__ void sum_partials_block(const double *partial, int n, double *dst)
{
    __shared__ double r[256];
    double a = 0.0;
    for (int k = threadIdx.x; k < n; k += 256) a += __ldcg(partial + k);
    r[threadIdx.x] = a;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) r[threadIdx.x] += r[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) *dst = r[0];
}

// ---------------------------------------------------------------------------
// Camera tables.  q = q(v) (x) q0 (compute_exQT.cl:82-87), M = matrix of
// X -> q (0,X) conj(q), D[m] = dM/dv_m through q(v) with s = sqrt(1-|v|^2).
// With cnp > 6 the intrinsics (fx, cx, cy, ar, skew) and, for cnp 16, the
// distortion (k1, k2, p1, p2, k3) are parameters 6.. of the camera, moved by
// dpa like the pose; with cnp 6 they come from the fixed K array.
// One lane per camera, six warps per block by role, so that no warp issues
// the whole table's FP64 instructions one after another (a warp issues one
// FP64 instruction per ~64 cycles): every warp forms q = q(v) (x) q0, then
// warp 0 writes M, t and the intrinsics (and their FP32 copy), warp 1 + m
// writes D[m] (only where the Jacobian is formed from the table: with_d),
// and warps 4 and 5 write the FP32-pair split of M and of t and the
// intrinsics (tab2f).
constexpr int CT_THREADS = 192;
__global__ void __launch_bounds__(CT_THREADS) k_cam_tables(int nc, int cnp, const double *__restrict__ K,
                                                           const double *__restrict__ q0,
                                                           const double *__restrict__ cams,
                                                           const double *__restrict__ dpa, double *__restrict__ tab,
                                                           float *__restrict__ tab32, float2 *__restrict__ tab2f,
                                                           int with_d)
{
    const int role = threadIdx.x >> 5;
    const int j = blockIdx.x * 32 + (threadIdx.x & 31);
    if (j >= nc) return;
    if ((role >= 1 && role <= 3 && !with_d) || (role >= 4 && !tab2f)) return;
    const double *cj = cams + (size_t)cnp * j;
    const double *dj = dpa ? dpa + (size_t)cnp * j : nullptr;
    // the translation and the intrinsics (roles 0 and 5)
    auto tk = [&](double (&t)[3], double (&kk)[5], double (&kc)[5]) {
        for (int m = 0; m < 3; ++m) t[m] = dj ? cj[3 + m] + dj[3 + m] : cj[3 + m];
        for (int m = 0; m < 5; ++m) kc[m] = 0.0;
        if (cnp > 6) {
            for (int m = 0; m < 5; ++m) kk[m] = dj ? cj[6 + m] + dj[6 + m] : cj[6 + m];
            if (cnp == 16)
                for (int m = 0; m < 5; ++m) kc[m] = dj ? cj[11 + m] + dj[11 + m] : cj[11 + m];
        } else {
            for (int m = 0; m < 5; ++m) kk[m] = K[5 * j + m];
        }
    };
    if (role == 5) {
        double t[3], kk[5], kc[5];
        tk(t, kk, kc);
        float2 *F = tab2f + (size_t)RES_TAB2F * j;
#pragma unroll
        for (int e = 0; e < 3; ++e) F[9 + e] = split2f(t[e]);
        F[12] = split2f(kk[0]);          // fx
        F[13] = split2f(kk[4]);          // sk
        F[14] = split2f(kk[1]);          // cx
        F[15] = split2f(kk[0] * kk[3]);  // fy
        F[16] = split2f(kk[2]);          // cy
        F[17] = make_float2(0.0f, 0.0f);
        return;
    }
    double vl[3];
    for (int m = 0; m < 3; ++m) vl[m] = dj ? cj[m] + dj[m] : cj[m];
    const double s0 = q0[4 * j], a1 = q0[4 * j + 1], a2 = q0[4 * j + 2], a3 = q0[4 * j + 3];
    const double sl = sqrt(1.0 - vl[0] * vl[0] - vl[1] * vl[1] - vl[2] * vl[2]);
    const double s = sl * s0 - (a1 * vl[0] + a2 * vl[1] + a3 * vl[2]);
    const double a = s0 * vl[0] + sl * a1 + a3 * vl[1] - a2 * vl[2];
    const double b = s0 * vl[1] + sl * a2 + a1 * vl[2] - a3 * vl[0];
    const double c = s0 * vl[2] + sl * a3 + a2 * vl[0] - a1 * vl[1];
    CamTab *T = reinterpret_cast<CamTab *>(tab + (size_t)CAMTAB * j);
    if (role == 0 || role == 4) {
        const double d = s * s - (a * a + b * b + c * c);
        const double M[9] = {d + 2 * a * a,       2 * (a * b - s * c), 2 * (a * c + s * b),
                             2 * (a * b + s * c), d + 2 * b * b,       2 * (b * c - s * a),
                             2 * (a * c - s * b), 2 * (b * c + s * a), d + 2 * c * c};
        if (role == 4) {  // the projection's rotation as FP32 pairs
            float2 *F = tab2f + (size_t)RES_TAB2F * j;
#pragma unroll
            for (int e = 0; e < 9; ++e) F[e] = split2f(M[e]);
            return;
        }
#pragma unroll
        for (int e = 0; e < 9; ++e) T->M[e] = M[e];
        if (tab32) {  // the mixed Jacobian's operands, rounded once per camera
            float *F = tab32 + (size_t)CAMTAB32 * j;
#pragma unroll
            for (int e = 0; e < 9; ++e) F[e] = (float)M[e];
        }
        double t[3], kk[5], kc[5];
        tk(t, kk, kc);
        for (int m = 0; m < 3; ++m) T->t[m] = t[m];
        T->fx = kk[0]; T->cx = kk[1]; T->cy = kk[2]; T->fy = kk[0] * kk[3]; T->sk = kk[4];
        if (tab32) {
            float *F = tab32 + (size_t)CAMTAB32 * j;
            F[36] = (float)T->fx;
            F[37] = (float)T->sk;
            F[38] = (float)T->fy;
            F[39] = 0.0f;
        }
        T->ar = kk[3];
        for (int m = 0; m < 5; ++m) T->kc[m] = kc[m];
        for (int m = 0; m < 6; ++m) T->pad[m] = 0.0;
        return;
    }
    // D[m] = dM/dv_m through q(v), with dM/d(s, a, b, c) and
    // dq/dv_m = (s0 ds - a0_m, a0 ds + s0 e_m + e_m x a0), ds = -v_m / s_l
    const int m = role - 1;
    const double dS[9] = {2 * s, -2 * c, 2 * b, 2 * c, 2 * s, -2 * a, -2 * b, 2 * a, 2 * s};
    const double dA[9] = {2 * a, 2 * b, 2 * c, 2 * b, -2 * a, -2 * s, 2 * c, 2 * s, -2 * a};
    const double dB[9] = {-2 * b, 2 * a, 2 * s, 2 * a, 2 * b, 2 * c, -2 * s, 2 * c, -2 * b};
    const double dC[9] = {-2 * c, -2 * s, 2 * a, 2 * s, -2 * c, 2 * b, 2 * a, 2 * b, 2 * c};
    const double vm = m == 0 ? vl[0] : m == 1 ? vl[1] : vl[2];
    const double am = m == 0 ? a1 : m == 1 ? a2 : a3;
    const double ds = -vm / sl;
    // e_m x a0
    const double x0 = m == 1 ? a3 : m == 2 ? -a2 : 0.0;
    const double x1 = m == 0 ? -a3 : m == 2 ? a1 : 0.0;
    const double x2 = m == 0 ? a2 : m == 1 ? -a1 : 0.0;
    const double dq0 = s0 * ds - am;
    const double dq1 = a1 * ds + (m == 0 ? s0 : 0.0) + x0;
    const double dq2 = a2 * ds + (m == 1 ? s0 : 0.0) + x1;
    const double dq3 = a3 * ds + (m == 2 ? s0 : 0.0) + x2;
    double *D = T->D + 9 * m;
#pragma unroll
    for (int e = 0; e < 9; ++e) D[e] = dS[e] * dq0 + dA[e] * dq1 + dB[e] * dq2 + dC[e] * dq3;
    if (tab32) {
        float *F = tab32 + (size_t)CAMTAB32 * j + 9 + 9 * m;
#pragma unroll
        for (int e = 0; e < 9; ++e) F[e] = (float)D[e];
    }
}

void launch_cam_tables(const DeviceProblem &d, const double *cams, const double *dpa, double *tab,
                       cudaStream_t s, float *tab32, float2 *tab2f, int with_d)
{
    k_cam_tables<<<ceil_div(d.nc, 32), CT_THREADS, 0, s>>>(d.nc, d.cnp, d.K, d.q0, cams, dpa, tab, tab32, tab2f,
                                                           with_d);
    note_launch(1);
}

// ---------------------------------------------------------------------------
// Linearization, one thread per observation: residual (compute_exQT.cl),
// Jacobian blocks A = d(x,y)/d(v,t), B = d(x,y)/dX (compute_jacobiQT.cl) by
// the chain rule through the camera table, and W = coeff A^T B
// (compute_Wblks.cl:28-33).
template <typename R>
__global__ void __launch_bounds__(256) k_linearize(int no, const int *__restrict__ obs_pt,
                                                   const int *__restrict__ obs_cam,
                                                   const double *__restrict__ meas,
                                                   const double *__restrict__ pts,
                                                   const double *__restrict__ tab, R coeff,
                                                   const double *__restrict__ wt,
                                                   R *__restrict__ ex, R *__restrict__ A,
                                                   R *__restrict__ B, R *__restrict__ W,
                                                   const float *__restrict__ tab32,
                                                   const float2 *__restrict__ meas2f,
                                                   const float2 *__restrict__ tab2f)
{
    int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= no) return;
    const int i = __ldg(obs_pt + o), j = __ldg(obs_cam + o);
    const double *T = tab + (size_t)CAMTAB * j;
    // e = m - pi(X) is a small difference of ~1e3 px quantities, and its error
    // moves the gradient and with it the LM fixed point, so the projection is
    // FP64 (the FP64 form, and the mixed form with covariance weights) or
    // double-float FP32 (the mixed form, unweighted: the point split here,
    // the measurements and camera table split into FP32 pairs once, ~2^-44
    // relative).  Only the stored e, J and W are rounded to R.  The mixed
    // form's table rows come in as 16-byte loads (the kernel is bound by the
    // issue of its global loads and stores, not by arithmetic).
    R X0, X1, X2, yc, iz, nu;
    double e0 = 0.0, e1 = 0.0, wa = 1.0, wb = 0.0, wc = 1.0;
    float e0f = 0.0f, e1f = 0.0f;
    const bool dfp = !is_fp64<R>() && tab2f != nullptr;
    if (dfp) {
        float2 Tf[RES_TAB2F];
        const float4 *T4 = reinterpret_cast<const float4 *>(tab2f + (size_t)RES_TAB2F * j);
#pragma unroll
        for (int k = 0; k < RES_TAB2F / 2; ++k) {
            const float4 q = __ldg(T4 + k);
            Tf[2 * k] = make_float2(q.x, q.y);
            Tf[2 * k + 1] = make_float2(q.z, q.w);
        }
        const df Xa = df_of(split2f(__ldg(pts + 3 * i))), Xb = df_of(split2f(__ldg(pts + 3 * i + 1))),
                 Xc = df_of(split2f(__ldg(pts + 3 * i + 2)));
        const df xc = df_add(df_add(df_mul(df_of(Tf[0]), Xa), df_mul(df_of(Tf[1]), Xb)),
                             df_add(df_mul(df_of(Tf[2]), Xc), df_of(Tf[9])));
        const df ycv = df_add(df_add(df_mul(df_of(Tf[3]), Xa), df_mul(df_of(Tf[4]), Xb)),
                              df_add(df_mul(df_of(Tf[5]), Xc), df_of(Tf[10])));
        const df zc = df_add(df_add(df_mul(df_of(Tf[6]), Xa), df_mul(df_of(Tf[7]), Xb)),
                             df_add(df_mul(df_of(Tf[8]), Xc), df_of(Tf[11])));
        const df izv = df_rcp(zc);
        const df nuv = df_add(df_mul(df_of(Tf[12]), xc), df_mul(df_of(Tf[13]), ycv));
        const df un = df_add(nuv, df_mul(df_of(Tf[14]), zc));
        const df vn = df_add(df_mul(df_of(Tf[15]), ycv), df_mul(df_of(Tf[16]), zc));
        const float4 m4 = __ldg(reinterpret_cast<const float4 *>(meas2f) + o);
        const df ea = df_add(df{m4.x, m4.y}, df_neg(df_mul(un, izv)));
        const df eb = df_add(df{m4.z, m4.w}, df_neg(df_mul(vn, izv)));
        e0f = __fadd_rn(ea.hi, ea.lo);
        e1f = __fadd_rn(eb.hi, eb.lo);
        X0 = (R)Xa.hi; X1 = (R)Xb.hi; X2 = (R)Xc.hi;
        yc = (R)__fadd_rn(ycv.hi, ycv.lo);
        iz = (R)__fadd_rn(izv.hi, izv.lo);
        nu = (R)__fadd_rn(nuv.hi, nuv.lo);
        st2<R>(ex + 2 * (size_t)o, (R)e0f, (R)e1f);
    } else {
        const double Xd0 = __ldg(pts + 3 * i), Xd1 = __ldg(pts + 3 * i + 1), Xd2 = __ldg(pts + 3 * i + 2);
        double Md[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) Md[e] = __ldg(T + e);
        const double xcd = Md[0] * Xd0 + Md[1] * Xd1 + Md[2] * Xd2 + __ldg(T + 36);
        const double ycd = Md[3] * Xd0 + Md[4] * Xd1 + Md[5] * Xd2 + __ldg(T + 37);
        const double zcd = Md[6] * Xd0 + Md[7] * Xd1 + Md[8] * Xd2 + __ldg(T + 38);
        const double fxd = __ldg(T + 39), skd = __ldg(T + 40), cxd = __ldg(T + 41), fyd = __ldg(T + 42),
                     cyd = __ldg(T + 43);
        const double izd = rcp_fast(zcd);
        const double2 m2 = __ldg(reinterpret_cast<const double2 *>(meas + 2 * (size_t)o));
        const double nud = fxd * xcd + skd * ycd;
        const double u = (nud + cxd * zcd) * izd;
        const double v = (fyd * ycd + cyd * zcd) * izd;
        e0 = m2.x - u;
        e1 = m2.y - v;
        if (wt) {  // whitening: e <- L e, J rows <- L J
            wa = __ldg(wt + 3 * (size_t)o);
            wb = __ldg(wt + 3 * (size_t)o + 1);
            wc = __ldg(wt + 3 * (size_t)o + 2);
            const double t0 = wa * e0 + wb * e1;
            e1 = wc * e1;
            e0 = t0;
        }
        st2<R>(ex + 2 * (size_t)o, (R)e0, (R)e1);
        X0 = (R)Xd0; X1 = (R)Xd1; X2 = (R)Xd2;
        yc = (R)ycd; iz = (R)izd; nu = (R)nud;
    }
    // the mixed form takes the table's FP32 copy (the same values, rounded
    // once per camera instead of once per observation on the FP64 pipe),
    // its 160-byte row in ten 16-byte loads
    float F[CAMTAB32];
    if constexpr (!is_fp64<R>()) {
        const float4 *F4 = reinterpret_cast<const float4 *>(tab32 + (size_t)CAMTAB32 * j);
#pragma unroll
        for (int k = 0; k < CAMTAB32 / 4; ++k) {
            const float4 q = __ldg(F4 + k);
            F[4 * k] = q.x;
            F[4 * k + 1] = q.y;
            F[4 * k + 2] = q.z;
            F[4 * k + 3] = q.w;
        }
    }
    R M[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) M[e] = is_fp64<R>() ? (R)__ldg(T + e) : (R)F[e];
    const R fx = is_fp64<R>() ? (R)__ldg(T + 39) : (R)F[36], sk = is_fp64<R>() ? (R)__ldg(T + 40) : (R)F[37],
            fy = is_fp64<R>() ? (R)__ldg(T + 42) : (R)F[38];
    // d(x,y)/dXc
    const R p00 = fx * iz, p01 = sk * iz, p02 = -nu * iz * iz;
    const R p11 = fy * iz, p12 = -fy * yc * iz * iz;
    // dXc/dv = D[m] X
    R a[12];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        R Dm[9];
        if constexpr (is_fp64<R>()) {
#pragma unroll
            for (int e = 0; e < 9; ++e) Dm[e] = __ldg(T + 9 + 9 * m + e);
        } else {
#pragma unroll
            for (int e = 0; e < 9; ++e) Dm[e] = F[9 + 9 * m + e];
        }
        const R g0 = Dm[0] * X0 + Dm[1] * X1 + Dm[2] * X2;
        const R g1 = Dm[3] * X0 + Dm[4] * X1 + Dm[5] * X2;
        const R g2 = Dm[6] * X0 + Dm[7] * X1 + Dm[8] * X2;
        a[m] = p00 * g0 + p01 * g1 + p02 * g2;
        a[6 + m] = p11 * g1 + p12 * g2;
    }
    a[3] = p00; a[4] = p01; a[5] = p02;
    a[9] = (R)0; a[10] = p11; a[11] = p12;
    R bb[6];
#pragma unroll
    for (int m = 0; m < 3; ++m) {
        bb[m] = p00 * M[m] + p01 * M[3 + m] + p02 * M[6 + m];
        bb[3 + m] = p11 * M[3 + m] + p12 * M[6 + m];
    }
    if (wt) {
        const R ra = (R)wa, rb = (R)wb, rc = (R)wc;
#pragma unroll
        for (int m = 0; m < 6; ++m) {
            const R a0 = a[m], a1 = a[6 + m];
            a[m] = ra * a0 + rb * a1;
            a[6 + m] = rc * a1;
        }
#pragma unroll
        for (int m = 0; m < 3; ++m) {
            const R b0 = bb[m], b1 = bb[3 + m];
            bb[m] = ra * b0 + rb * b1;
            bb[3 + m] = rc * b1;
        }
    }
    if constexpr (is_fp64<R>()) {
        stn<R, 12>(A + 12 * (size_t)o, a);
    } else {  // a 48-byte row: three 16-byte stores
        float4 *A4 = reinterpret_cast<float4 *>(A + 12 * (size_t)o);
#pragma unroll
        for (int k = 0; k < 3; ++k) A4[k] = make_float4(a[4 * k], a[4 * k + 1], a[4 * k + 2], a[4 * k + 3]);
    }
    stn<R, 6>(B + 6 * (size_t)o, bb);
    // W with coeff folded into a copy of B: the solver's coeff is 1 or 2, a
    // power of two, so coeff (a b + a' b') and a (coeff b) + a' (coeff b') are
    // the same number.  The y row of A has a zero for t_x (a[9], also after
    // whitening, whose factor is triangular), so row 3 takes one product.
    R cb[6];
#pragma unroll
    for (int m = 0; m < 6; ++m) cb[m] = coeff * bb[m];
    R w[18];
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) w[r * 3 + c] = r == 3 ? a[3] * cb[c] : a[r] * cb[c] + a[6 + r] * cb[3 + c];
    stn<R, 18>(W + 18 * (size_t)o, w);
}

void launch_linearize(const DeviceProblem &d, double coeff, cudaStream_t s)
{
    if (d.cnp != 6) return launch_linearize_v(d, coeff, s);
    if (d.no == 0) return;
    if (d.prec == PSBA_PREC_FP64) {
        k_linearize<double><<<ceil_div(d.no, 256), 256, 0, s>>>(d.no, d.obs_pt, d.obs_cam, d.meas, d.pts,
                                                                  d.camtab, coeff, d.wt, d.ex, d.A, d.B, d.W,
                                                                  nullptr, nullptr, nullptr);
    } else {
        // unweighted: the double-float projection from the table's split
        // (k_cam_tables of this linearization)
        const bool dfp = linearize_df(d);
        k_linearize<float><<<ceil_div(d.no, 256), 256, 0, s>>>(
            d.no, d.obs_pt, d.obs_cam, d.meas, d.pts, d.camtab, (float)coeff, d.wt, (float *)d.ex, (float *)d.A,
            (float *)d.B, (float *)d.W, d.camtab32, dfp ? d.meas2f : nullptr, dfp ? d.tab2f : nullptr);
    }
    note_launch(1);
}

// ---------------------------------------------------------------------------
// Residual and its squared norm at (camera table, pts [+ dpb]); block partials.
// The 17 table values the projection uses (rotation, translation, K) are
// staged per block in shared memory when the cameras fit (stage_nc > 0):
// neighbouring observations belong to different cameras, so reading them
// from the table makes every load of a warp touch up to 32 cache lines.
constexpr int RES_TAB = 17;  // M (9), t (3), fx sk cx fy cy (5)

__device__ __forceinline__ int res_tab_src(int k) { return k < 9 ? k : 36 + (k - 9); }

__global__ void __launch_bounds__(256) k_residual(int no, const int *__restrict__ obs_pt,
                                                  const int *__restrict__ obs_cam,
                                                  const double *__restrict__ meas,
                                                  const double *__restrict__ pts,
                                                  const double *__restrict__ dpb,
                                                  const double *__restrict__ tab,
                                                  const double *__restrict__ wt,
                                                  double *__restrict__ ex_out,
                                                  double *__restrict__ partial, int stage_nc,
                                                  double *__restrict__ sum_dst, int *__restrict__ ticket)
{
    __shared__ double red[256 / 32];
    extern __shared__ double s_tab[];  // stage_nc * RES_TAB
    for (int e = threadIdx.x; e < stage_nc * RES_TAB; e += blockDim.x)
        s_tab[e] = __ldg(tab + (size_t)CAMTAB * (e / RES_TAB) + res_tab_src(e % RES_TAB));
    if (stage_nc > 0) __syncthreads();
    // a few resident blocks per SM, each thread over the observations o, o +
    // the grid's threads, ...: the table is staged once per block instead of
    // once per 256 observations; each thread's squares summed in its order
    double sq = 0.0;
#pragma unroll 2
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < no; o += gridDim.x * blockDim.x) {
        const int i = __ldg(obs_pt + o), j = __ldg(obs_cam + o);
        double X[3];
#pragma unroll
        for (int m = 0; m < 3; ++m)
            X[m] = dpb ? __ldg(pts + 3 * i + m) + __ldg(dpb + 3 * i + m) : __ldg(pts + 3 * i + m);
        double Tv[RES_TAB];
        if (stage_nc > 0) {
#pragma unroll
            for (int k = 0; k < RES_TAB; ++k) Tv[k] = s_tab[j * RES_TAB + k];
        } else {
            const double *T = tab + (size_t)CAMTAB * j;
#pragma unroll
            for (int k = 0; k < RES_TAB; ++k) Tv[k] = __ldg(T + res_tab_src(k));
        }
        const double xc = Tv[0] * X[0] + Tv[1] * X[1] + Tv[2] * X[2] + Tv[9];
        const double yc = Tv[3] * X[0] + Tv[4] * X[1] + Tv[5] * X[2] + Tv[10];
        const double zc = Tv[6] * X[0] + Tv[7] * X[1] + Tv[8] * X[2] + Tv[11];
        const double iz = rcp_fast(zc);
        const double u = (Tv[12] * xc + Tv[13] * yc + Tv[14] * zc) * iz;
        const double v = (Tv[15] * yc + Tv[16] * zc) * iz;
        const double2 m2 = __ldg(reinterpret_cast<const double2 *>(meas + 2 * (size_t)o));
        double e0 = m2.x - u, e1 = m2.y - v;
        if (wt) {
            const double t0 = wt[3 * (size_t)o] * e0 + wt[3 * (size_t)o + 1] * e1;
            e1 = wt[3 * (size_t)o + 2] * e1;
            e0 = t0;
        }
        if (ex_out) *reinterpret_cast<double2 *>(ex_out + 2 * (size_t)o) = make_double2(e0, e1);
        sq = fma(e0, e0, fma(e1, e1, sq));
    }
    // fixed-order block sum: xor tree in each warp, then the warps in order
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = red[0];
        for (int w = 1; w < 256 / 32; ++w) a += red[w];
        partial[blockIdx.x] = a;
    }
    if (sum_dst && take_last_ticket(ticket)) {
        sum_partials_block(partial, gridDim.x, sum_dst);
        if (threadIdx.x == 0) *ticket = 0;
    }
}

// The mixed form's trial cost (unweighted, 6-parameter cameras): the same
// projection and sum of squares as k_residual, in double-float FP32
// arithmetic from the trial camera table and trial points split once into
// FP32 pairs (k_cam_tables, k_eb_dpb) and the measurements split once per
// handle.  The residual e = m - pi(X) of ~1 px is a difference of ~1e3 px
// values; its double-float error is ~1e3 * 2^-44 px, far below what the gain
// ratio resolves, and no FP64 instruction is issued per observation (each
// thread converts its sum once).
__global__ void __launch_bounds__(256) k_residual_df(int no, int nc, const int *__restrict__ obs_pt,
                                                     const int *__restrict__ obs_cam,
                                                     const float2 *__restrict__ meas2f,
                                                     const float2 *__restrict__ x2f,
                                                     const float2 *__restrict__ tab2f, double *__restrict__ partial,
                                                     double *__restrict__ sum_dst, int *__restrict__ ticket)
{
    __shared__ double red[256 / 32];
    extern __shared__ float2 s_tab2[];  // nc * RES_TAB2F
    for (int e = threadIdx.x; e < nc * RES_TAB2F; e += blockDim.x) s_tab2[e] = tab2f[e];
    __syncthreads();
    df sq{0.0f, 0.0f};
    for (int o = blockIdx.x * blockDim.x + threadIdx.x; o < no; o += gridDim.x * blockDim.x) {
        const int i = __ldg(obs_pt + o), j = __ldg(obs_cam + o);
        const float2 *T = s_tab2 + RES_TAB2F * j;
        const df X0 = df_of(__ldg(x2f + 3 * (size_t)i)), X1 = df_of(__ldg(x2f + 3 * (size_t)i + 1)),
                 X2 = df_of(__ldg(x2f + 3 * (size_t)i + 2));
        const df xc = df_add(df_add(df_mul(df_of(T[0]), X0), df_mul(df_of(T[1]), X1)),
                             df_add(df_mul(df_of(T[2]), X2), df_of(T[9])));
        const df yc = df_add(df_add(df_mul(df_of(T[3]), X0), df_mul(df_of(T[4]), X1)),
                             df_add(df_mul(df_of(T[5]), X2), df_of(T[10])));
        const df zc = df_add(df_add(df_mul(df_of(T[6]), X0), df_mul(df_of(T[7]), X1)),
                             df_add(df_mul(df_of(T[8]), X2), df_of(T[11])));
        const df iz = df_rcp(zc);
        const df un = df_add(df_add(df_mul(df_of(T[12]), xc), df_mul(df_of(T[13]), yc)), df_mul(df_of(T[14]), zc));
        const df vn = df_add(df_mul(df_of(T[15]), yc), df_mul(df_of(T[16]), zc));
        const df e0 = df_add(df_of(__ldg(meas2f + 2 * (size_t)o)), df_neg(df_mul(un, iz)));
        const df e1 = df_add(df_of(__ldg(meas2f + 2 * (size_t)o + 1)), df_neg(df_mul(vn, iz)));
        sq = df_add(sq, df_add(df_mul(e0, e0), df_mul(e1, e1)));
    }
    double x = (double)sq.hi + (double)sq.lo;
    // fixed-order block sum: xor tree in each warp, then the warps in order
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(0xffffffffu, x, off);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = red[0];
        for (int w = 1; w < 256 / 32; ++w) a += red[w];
        partial[blockIdx.x] = a;
    }
    if (take_last_ticket(ticket)) {
        sum_partials_block(partial, gridDim.x, sum_dst);
        if (threadIdx.x == 0) *ticket = 0;
    }
}

void launch_residual_df(const DeviceProblem &d, double *partial, int nblocks, double *sum_dst, cudaStream_t s)
{
    k_residual_df<<<nblocks, 256, sizeof(float2) * RES_TAB2F * d.nc, s>>>(
        d.no, d.nc, d.obs_pt, d.obs_cam, d.meas2f, d.x2f, d.tab2f, partial, sum_dst, d.tickets + 1);
    note_launch(1);
}

__global__ void k_split2f(const double *__restrict__ x, float2 *__restrict__ out, long long n)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) out[i] = split2f(x[i]);
}

void launch_split2f(const double *x, float2 *out, long long n, cudaStream_t s)
{
    if (n <= 0) return;
    k_split2f<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(x, out, n);
    note_launch(1);
}

// cameras whose residual-table values a block stages (0: read the table)
int residual_stage_nc(const DeviceProblem &d)
{
    return (size_t)d.nc * RES_TAB * sizeof(double) <= 48 * 1024 ? d.nc : 0;
}

// k_residual's grid: four blocks of 256 per SM at most (its loop takes the rest)
int residual_blocks(const DeviceProblem &d)
{
    static std::mutex mu;
    static int sms_dev[MAX_DEVICES] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= MAX_DEVICES) dev = 0;
    int sms = 0;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (sms_dev[dev] == 0) cudaDeviceGetAttribute(&sms_dev[dev], cudaDevAttrMultiProcessorCount, dev);
        sms = std::max(1, sms_dev[dev]);
    }
    return std::max(1, std::min(ceil_div(d.no > 0 ? d.no : 1, 256), 4 * sms));
}

void launch_residual(const DeviceProblem &d, const double *tab, const double *pts, const double *dpb,
                     double *ex_out, double *partial, int nblocks, double *sum_dst, cudaStream_t s)
{
    if (d.cnp == 16) {
        launch_residual_dist(d, tab, pts, dpb, ex_out, partial, nblocks, s);
        launch_sum_partials(partial, nblocks, sum_dst, s);
        return;
    }
    const int snc = residual_stage_nc(d);
    k_residual<<<nblocks, 256, sizeof(double) * RES_TAB * snc, s>>>(d.no, d.obs_pt, d.obs_cam, d.meas, pts, dpb,
                                                                    tab, d.wt, ex_out, partial, snc, sum_dst,
                                                                    d.tickets + 1);
    note_launch(1);
}


// ---------------------------------------------------------------------------
// Per-point sums: V_i = coeff sum B^T B (compute_V.cl:24-37) and
// gb_i = coeff sum B^T e (compute_g.cl:42-57): 3 m lanes a point, each
// summing every (3 m)-th observation in ascending camera order, then the
// lanes' sums added in a fixed order.
// V is accumulated to FP64 accuracy in both forms (in the mixed form from
// FP32 products, in double-float FP32 arithmetic: ~2^-44 of the terms): an
// FP32 running sum of B^T B can turn the nearly singular V of a point seen
// from two close cameras indefinite, which moved the mixed form's LM fixed
// point by 7e-3 of the cost on a 24-camera power-law scene.
template <typename R>
__global__ void __launch_bounds__(256) k_point_blocks(int np, int ncp, const int2 *__restrict__ eb_warps,
                                                      const int *__restrict__ pt_start,
                                                      const int *__restrict__ pt_order, const R *__restrict__ B,
                                                      const R *__restrict__ ex, R coeff, double *__restrict__ V,
                                                      double *__restrict__ g, double *__restrict__ uvdiag,
                                                      float *__restrict__ gb32)
{
    // the eb/dpb warp schedule (points in pt_order, 3 m lanes a point): lane
    // r of a point sums its observations r, r + L, r + 2L, ... (L = 3 m), so
    // no lane walks more than ~4 of them; lane 0 then adds the L partial sums
    // in order of r
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int2 wi = eb_warps[blockIdx.x * EB_WARPS + warp];
    const int npw = eb_warps[blockIdx.x * EB_WARPS + warp + 1].x - wi.x;
    const int L = 3 * wi.y, pw = lane / L, r = lane - L * pw;
    const bool live = pw < npw;
    const int i = live ? pt_order[wi.x + pw] : 0;
    double a[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};  // v00 v01 v02 v11 v12 v22, then the gradient
    if constexpr (is_fp64<R>()) {
        if (live) {
            const int e = pt_start[i + 1];
#pragma unroll 2
            for (int o = pt_start[i] + r; o < e; o += L) {
                R b[6], ee[2];
                ldn<R, 6>(B + 6 * (size_t)o, b);
                ld2<R>(ex + 2 * (size_t)o, ee[0], ee[1]);
                const R b0 = b[0], b1 = b[1], b2 = b[2], c0 = b[3], c1 = b[4], c2 = b[5];
                const R e0 = ee[0], e1 = ee[1];
                a[0] = a[0] + b0 * b0 + c0 * c0;
                a[1] = a[1] + b0 * b1 + c0 * c1;
                a[2] = a[2] + b0 * b2 + c0 * c2;
                a[3] = a[3] + b1 * b1 + c1 * c1;
                a[4] = a[4] + b1 * b2 + c1 * c2;
                a[5] = a[5] + b2 * b2 + c2 * c2;
                a[6] = a[6] + b0 * e0 + c0 * e1;
                a[7] = a[7] + b1 * e0 + c1 * e1;
                a[8] = a[8] + b2 * e0 + c2 * e1;
            }
        }
    } else {
        // the mixed form in double-float FP32 arithmetic (hi, lo pairs,
        // TwoSum), converted to FP64 once per lane: V sums the FP32 products
        // b_k b_l + c_k c_l, the gradient the exact products b e (each split
        // by an FMA), so the sums are those of FP64 to ~2^-44 without an FP64
        // instruction per observation
        float h[9], l[9];
#pragma unroll
        for (int v = 0; v < 9; ++v) h[v] = l[v] = 0.0f;
        if (live) {
            const int e = pt_start[i + 1];
            for (int o = pt_start[i] + r; o < e; o += L) {
                float b[6], e0, e1;
                ldn<float, 6>(reinterpret_cast<const float *>(B) + 6 * (size_t)o, b);
                ld2<float>(reinterpret_cast<const float *>(ex) + 2 * (size_t)o, e0, e1);
                const float vv[6] = {fmaf(b[0], b[0], b[3] * b[3]), fmaf(b[0], b[1], b[3] * b[4]),
                                     fmaf(b[0], b[2], b[3] * b[5]), fmaf(b[1], b[1], b[4] * b[4]),
                                     fmaf(b[1], b[2], b[4] * b[5]), fmaf(b[2], b[2], b[5] * b[5])};
#pragma unroll
                for (int v = 0; v < 6; ++v) {
                    float t;
                    two_sum_f(h[v], vv[v], h[v], t);
                    l[v] += t;
                }
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float p0 = __fmul_rn(b[k], e0), p1 = __fmul_rn(b[3 + k], e1);
                    const float q = fmaf(b[k], e0, -p0) + fmaf(b[3 + k], e1, -p1);
                    float t0, t1;
                    two_sum_f(h[6 + k], p0, h[6 + k], t0);
                    two_sum_f(h[6 + k], p1, h[6 + k], t1);
                    l[6 + k] += (t0 + t1) + q;
                }
            }
        }
        // the L lanes' sums meet in double-float too, in order of r (lane 0
        // of the point collects), and the nine totals are converted to FP64
        // by the point's L lanes, a few each: FP64 work per warp ~3 x 4
        // instructions instead of ~9 L
        // (each lane's own sums are what is exchanged, not running sums)
        float sh[9], sl[9];
#pragma unroll
        for (int v = 0; v < 9; ++v) {
            sh[v] = h[v];
            sl[v] = l[v];
        }
        for (int q = 1; q < L; ++q) {
            const int src = min(L * pw + q, 31);
#pragma unroll
            for (int v = 0; v < 9; ++v) {
                const float oh = __shfl_sync(0xffffffffu, h[v], src);
                const float ol = __shfl_sync(0xffffffffu, l[v], src);
                float t;
                two_sum_f(sh[v], oh, sh[v], t);
                sl[v] += ol + t;
            }
        }
        const int head = min(L * pw, 31);
#pragma unroll
        for (int v = 0; v < 9; ++v) {
            h[v] = __shfl_sync(0xffffffffu, sh[v], head);
            l[v] = __shfl_sync(0xffffffffu, sl[v], head);
        }
        if (!live) return;
        const double cf = (double)coeff;
#pragma unroll
        for (int j = 0; j < 3; ++j) {  // L >= 3: value r + j L
            const int v = r + j * L;
            if (v >= 9) break;
            float hv = h[0], lv = l[0];
#pragma unroll
            for (int u = 1; u < 9; ++u)
                if (u == v) {
                    hv = h[u];
                    lv = l[u];
                }
            const double x = cf * ((double)hv + (double)lv);
            if (v < 6) {
                V[6 * (size_t)i + v] = x;
                if (v == 0 || v == 3 || v == 5) uvdiag[ncp + 3 * (size_t)i + (v == 0 ? 0 : v == 3 ? 1 : 2)] = x;
            } else {
                g[ncp + 3 * (size_t)i + (v - 6)] = x;
                if (gb32) gb32[3 * (size_t)i + (v - 6)] = (float)x;  // the mixed form's ea sums take gb in FP32
            }
        }
        return;
    }
    if constexpr (is_fp64<R>()) {
        double s[9];
#pragma unroll
        for (int v = 0; v < 9; ++v) s[v] = a[v];
        for (int q = 1; q < L; ++q) {  // L is the same for the whole warp
            const int src = min(L * pw + q, 31);
#pragma unroll
            for (int v = 0; v < 9; ++v) s[v] += __shfl_sync(0xffffffffu, a[v], src);
        }
        if (!live || r != 0) return;
        const double cf = (double)coeff;
        double *Vi = V + 6 * (size_t)i;
        Vi[0] = cf * s[0]; Vi[1] = cf * s[1]; Vi[2] = cf * s[2];
        Vi[3] = cf * s[3]; Vi[4] = cf * s[4]; Vi[5] = cf * s[5];
        uvdiag[ncp + 3 * (size_t)i] = Vi[0];
        uvdiag[ncp + 3 * (size_t)i + 1] = Vi[3];
        uvdiag[ncp + 3 * (size_t)i + 2] = Vi[5];
        g[ncp + 3 * (size_t)i] = cf * s[6];
        g[ncp + 3 * (size_t)i + 1] = cf * s[7];
        g[ncp + 3 * (size_t)i + 2] = cf * s[8];
    }
}

void launch_point_blocks(const DeviceProblem &d, double coeff, cudaStream_t s)
{
    if (d.np == 0) return;
    if (d.prec == PSBA_PREC_FP64)
        k_point_blocks<double><<<eb_blocks(d), 256, 0, s>>>(d.np, d.N, d.eb_warps, d.pt_start, d.pt_order, d.B,
                                                              d.ex, coeff, d.V, d.g, d.uvdiag, nullptr);
    else
        k_point_blocks<float><<<eb_blocks(d), 256, 0, s>>>(d.np, d.N, d.eb_warps, d.pt_start, d.pt_order,
                                                             (const float *)d.B, (const float *)d.ex, (float)coeff,
                                                             d.V, d.g, d.uvdiag, d.cnp == 6 ? d.gb32 : nullptr);
    note_launch(1);
}

// ---------------------------------------------------------------------------
// Per-camera sums U_j = coeff sum A^T A (compute_U.cl:21-34) and
// ga_j = coeff sum A^T e (compute_g.cl:25-41) over the camera-sorted list,
// split in units of CAM_SUPER observations; a fixed-order sum per unit,
// then the units summed in order.
constexpr int CAM_THREADS = 128;
constexpr int CAM_NV = 27;  // 21 upper-triangle entries of A^T A + 6 of A^T e
static_assert(CAM_SUPER == CAM_THREADS * CAM_PER, "camera unit size");

// One CTA per unit of <= CAM_SUPER observations of a camera, CAM_PER
// consecutive observations a thread (FP64: accumulated directly; FP32: the
// products summed over the thread's observations, then one FP64 addition);
// the CTA then sums its threads' partials in a fixed order, each output by
// four threads over 32 partials, then the four.
template <typename R>
__global__ void __launch_bounds__(CAM_THREADS, 1) k_camera_partial(const CamUnit *__restrict__ units,
                                                                const int *__restrict__ cam_obs,
                                                                const R *__restrict__ A,
                                                                const R *__restrict__ ex,
                                                                double *__restrict__ partial)
{
    static_assert(CAM_THREADS == 128 && CAM_NV * 4 <= CAM_THREADS && CAM_PER <= FLUSH, "camera unit layout");
    __shared__ double red[CAM_NV][CAM_THREADS + 1];
    const CamUnit u = units[blockIdx.x];
    const int t = threadIdx.x;
    double acc[CAM_NV];
#pragma unroll
    for (int v = 0; v < CAM_NV; ++v) acc[v] = 0.0;
    R part[21];
#pragma unroll
    for (int v = 0; v < 21; ++v) part[v] = (R)0;
    float gh[6], gl[6];  // mixed form: the gradient sums as double-float pairs
#pragma unroll
    for (int q = 0; q < 6; ++q) gh[q] = gl[q] = 0.0f;
    const int k0 = t * CAM_PER, k1 = min(u.count, k0 + CAM_PER);
    if constexpr (is_fp64<R>()) {
        for (int kk = k0; kk < k1; ++kk) {
            const int o = __ldg(cam_obs + u.begin + kk);
            R a[12], e2[2];
            ldn<R, 12>(A + 12 * (size_t)o, a);
            ld2<R>(ex + 2 * (size_t)o, e2[0], e2[1]);
            int v = 0;
#pragma unroll
            for (int r = 0; r < 6; ++r)
#pragma unroll
                for (int c = r; c < 6; ++c, ++v) acc[v] = acc[v] + a[r] * a[c] + a[6 + r] * a[6 + c];
            // the gradient sets the LM fixed point: sums of the exact
            // products of the stored values
#pragma unroll
            for (int q = 0; q < 6; ++q) acc[21 + q] = acc[21 + q] + a[q] * e2[0] + a[6 + q] * e2[1];
        }
    } else {
        // the mixed form: the thread's indices first, then its rows four at
        // a time (48-byte A rows as three 16-byte loads), so that up to four
        // gathered rows are in flight at once; summed in the same order
        int oo[CAM_PER];
#pragma unroll
        for (int q = 0; q < CAM_PER; ++q) oo[q] = k0 + q < k1 ? __ldg(cam_obs + u.begin + k0 + q) : -1;
#pragma unroll
        for (int q0 = 0; q0 < CAM_PER; q0 += 4) {
            float a4[4][12], e4[4][2];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (oo[q0 + q] < 0) continue;
                const float4 *A4 = reinterpret_cast<const float4 *>(A + 12 * (size_t)oo[q0 + q]);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const float4 x = __ldg(A4 + k);
                    a4[q][4 * k] = x.x;
                    a4[q][4 * k + 1] = x.y;
                    a4[q][4 * k + 2] = x.z;
                    a4[q][4 * k + 3] = x.w;
                }
                ld2<float>(ex + 2 * (size_t)oo[q0 + q], e4[q][0], e4[q][1]);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (oo[q0 + q] < 0) continue;
                const float *a = a4[q];
                int v = 0;
#pragma unroll
                for (int r = 0; r < 6; ++r)
#pragma unroll
                    for (int c = r; c < 6; ++c, ++v) part[v] = part[v] + a[r] * a[c] + a[6 + r] * a[6 + c];
                // the gradient sets the LM fixed point: sums of the exact
                // products of the stored values in double-float FP32
                // arithmetic (each product split by an FMA, TwoSum, to ~2^-44
                // of the terms)
#pragma unroll
                for (int k = 0; k < 6; ++k) {
                    const float p0 = __fmul_rn(a[k], e4[q][0]), p1 = __fmul_rn(a[6 + k], e4[q][1]);
                    const float r = fmaf(a[k], e4[q][0], -p0) + fmaf(a[6 + k], e4[q][1], -p1);
                    float t0, t1;
                    two_sum_f(gh[k], p0, gh[k], t0);
                    two_sum_f(gh[k], p1, gh[k], t1);
                    gl[k] += (t0 + t1) + r;
                }
            }
        }
    }
    if constexpr (!is_fp64<R>()) {
        // the mixed form sums the threads' values in double-float FP32
        // arithmetic too (the same fixed order), converting only the 27
        // totals: no FP64 instruction per thread
        float2(*red2)[CAM_THREADS + 1] = reinterpret_cast<float2(*)[CAM_THREADS + 1]>(red);
#pragma unroll
        for (int v = 0; v < 21; ++v) red2[v][t] = make_float2(part[v], 0.0f);
#pragma unroll
        for (int q = 0; q < 6; ++q) red2[21 + q][t] = make_float2(gh[q], gl[q]);
        __syncthreads();
        float sh = 0.0f, sl = 0.0f;
        const int v = t >> 2, g = t & 3;
        if (v < CAM_NV) {
#pragma unroll 8
            for (int q = 0; q < CAM_THREADS / 4; ++q) {
                const float2 x = red2[v][g * (CAM_THREADS / 4) + q];
                float e;
                two_sum_f(sh, x.x, sh, e);
                sl += x.y + e;
            }
        }
        __syncthreads();
        if (v < CAM_NV) red2[v][g] = make_float2(sh, sl);
        __syncthreads();
        if (t < CAM_NV) {
            float h = red2[t][0].x, l = red2[t][0].y;
#pragma unroll
            for (int q = 1; q < 4; ++q) {
                float e;
                two_sum_f(h, red2[t][q].x, h, e);
                l += red2[t][q].y + e;
            }
            partial[(size_t)blockIdx.x * CAM_NV + t] = (double)h + (double)l;
        }
    } else {
#pragma unroll
        for (int v = 0; v < CAM_NV; ++v) red[v][t] = acc[v];
        __syncthreads();
        double s = 0.0;
        const int v = t >> 2, g = t & 3;
        if (v < CAM_NV) {
#pragma unroll 8
            for (int q = 0; q < CAM_THREADS / 4; ++q) s += red[v][g * (CAM_THREADS / 4) + q];
        }
        __syncthreads();
        if (v < CAM_NV) red[v][g] = s;
        __syncthreads();
        if (t < CAM_NV)
            partial[(size_t)blockIdx.x * CAM_NV + t] = (red[t][0] + red[t][1]) + (red[t][2] + red[t][3]);
    }
}

__global__ void k_camera_finish(int nc, const int *__restrict__ unit_start,
                                const double *__restrict__ partial, double coeff,
                                double *__restrict__ U, double *__restrict__ g,
                                double *__restrict__ uvdiag)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    if (id >= nc * CAM_NV) return;
    const int j = id / CAM_NV, v = id % CAM_NV;
    double sum = 0.0;
    for (int u = unit_start[j]; u < unit_start[j + 1]; ++u) sum += partial[(size_t)u * CAM_NV + v];
    sum = coeff * sum;
    if (v >= 21) {
        g[6 * j + (v - 21)] = sum;
        return;
    }
    // v -> (r, c), r <= c, row-major over the upper triangle
    int r = 0, c = 0, k = v;
    for (r = 0; r < 6; ++r) {
        if (k < 6 - r) {
            c = r + k;
            break;
        }
        k -= 6 - r;
    }
    U[36 * (size_t)j + r * 6 + c] = sum;
    U[36 * (size_t)j + c * 6 + r] = sum;
    if (r == c) uvdiag[6 * j + r] = sum;
}

void launch_camera_blocks(const DeviceProblem &d, double coeff, cudaStream_t s)
{
    if (d.cnp != 6) return launch_camera_blocks_v(d, coeff, s);
    if (d.n_cam_units > 0) {
        if (d.prec == PSBA_PREC_FP64)
            k_camera_partial<double><<<d.n_cam_units, CAM_THREADS, 0, s>>>(d.cam_units, d.cam_obs, d.A, d.ex,
                                                                             d.cam_partial);
        else
            k_camera_partial<float><<<d.n_cam_units, CAM_THREADS, 0, s>>>(
                d.cam_units, d.cam_obs, (const float *)d.A, (const float *)d.ex, d.cam_partial);
        note_launch(1);
    }
    k_camera_finish<<<ceil_div(d.nc * CAM_NV, 128), 128, 0, s>>>(d.nc, d.cam_unit_start,
                                                                   d.cam_partial, coeff, d.U, d.g,
                                                                   d.uvdiag); note_launch(1);
}

// ---------------------------------------------------------------------------
// V_i^-1 of the damped V_i + mu I by cofactors (compute_Vinv.cl:29-86); the
// near-singular branch (|T| < 1e-16, :31-73) restates the reference's pivoted
// elimination on the symmetric matrix.
template <typename R, bool FAST = false>
__device__ __forceinline__ void vinv_one(const R *Vi, R mu, R *out)
{
    const R a11 = Vi[0] + mu, a12 = Vi[1], a13 = Vi[2], a22 = Vi[3] + mu, a23 = Vi[4],
            a33 = Vi[5] + mu;
    R T = (a33 * a12 * a12 - 2 * a12 * a13 * a23 + a22 * a13 * a13 + a11 * a23 * a23 -
                a11 * a22 * a33);
    if (fabs(T) < (R)1e-16) {
        const R a21 = a12, a31 = a13, a32 = a23;
        R m[3][3] = {{a11, a12, a13}, {a21, a22, a23}, {a31, a32, a33}}, tmp;
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
        if (m[1][1] != (R)0) {
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
    if constexpr (FAST) {
        // the mixed form: one reciprocal (within 1 ulp of 1 / T in this
        // range) and six products instead of six divisions
        if (fabs(T) > 0x1p-80 && fabs(T) < 0x1p80) {
            const R iT = -rcp_fast(T);
            out[0] = (-a23 * a23 + a22 * a33) * iT;
            out[1] = (a13 * a23 - a12 * a33) * iT;
            out[2] = (a12 * a23 - a13 * a22) * iT;
            out[3] = (-a13 * a13 + a11 * a33) * iT;
            out[4] = (a12 * a13 - a11 * a23) * iT;
            out[5] = (-a12 * a12 + a11 * a22) * iT;
            return;
        }
    }
    out[0] = -(-a23 * a23 + a22 * a33) / T;
    out[1] = -(a13 * a23 - a12 * a33) / T;
    out[2] = -(a12 * a23 - a13 * a22) / T;
    out[3] = -(-a13 * a13 + a11 * a33) / T;
    out[4] = -(a12 * a13 - a11 * a23) / T;
    out[5] = -(-a12 * a12 + a11 * a22) / T;
}

// The damping is added and the inverse taken in FP64 in both forms (the mixed
// form multiplies by one reciprocal of the determinant where the FP64 form,
// like the reference, divides six times), and V^-1
// is kept in FP64: for a point seen from two nearby cameras V_i is nearly
// singular, and an FP32 V_i + mu I (which drops mu) or an FP32 V^-1 moves the
// LM fixed point by ~1e-2 of the cost.
// Each damping trial starts here, so this launch also clears the status word
// of the trial's bulk copies (status[2], set by k_yblocks_bulk when a wait
// runs out), which nothing else resets.
__global__ void k_vinv(int np, const double *__restrict__ V, double mu, double *__restrict__ Vinv,
                       float *__restrict__ Vinv2f, int *__restrict__ status)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0) status[2] = 0;
    if (i >= np) return;
    double vi[6], out[6];
#pragma unroll
    for (int e = 0; e < 6; ++e) vi[e] = V[6 * (size_t)i + e];
    if (Vinv2f)
        vinv_one<double, true>(vi, mu, out);
    else
        vinv_one<double>(vi, mu, out);
#pragma unroll
    for (int e = 0; e < 6; ++e) Vinv[6 * (size_t)i + e] = out[e];
    if (Vinv2f) {  // hi = fl32(v), lo = fl32(v - hi): v to ~2^-48
        float2 *dst = reinterpret_cast<float2 *>(Vinv2f + 12 * (size_t)i);
#pragma unroll
        for (int e = 0; e < 6; ++e) {
            const float hi = (float)out[e];
            dst[e] = make_float2(hi, (float)(out[e] - (double)hi));
        }
    }
}

void launch_vinv(const DeviceProblem &d, double mu, cudaStream_t s)
{
    if (d.np == 0) return;
    k_vinv<<<ceil_div(d.np, 128), 128, 0, s>>>(d.np, d.V, mu, d.Vinv,
                                               d.prec == PSBA_PREC_MIXED && d.cnp == 6 ? d.Vinv2f : nullptr,
                                               d.status);
    note_launch(1);
}



// Y = W V^-1 (compute_Yblks.cl:26-37), one thread per observation, the
// mixed form: W in FP32, V^-1 inverted in FP64 and carried as FP32 pairs
// (hi + lo, split once per point), each Y entry formed in double-float
// arithmetic and rounded to FP32.  No value passes through the FP64 pipe (on
// GB300 a conversion between FP32 and FP64 issues there), and Y keeps the
// accuracy of an FP64 product: a V^-1 rounded to FP32 instead breaks it for
// points seen from nearby cameras (V nearly singular, V^-1 with large entries
// of both signs), which sent LM to minima ~3% higher.  The FP64 form is
// k_yblocks_bulk.
__global__ void __launch_bounds__(256) k_yblocks(int no, const int *__restrict__ obs_pt,
                                                 const float *__restrict__ W, const float *__restrict__ Vinv2f,
                                                 float *__restrict__ Y)
{
    // a warp's 32 rows (2,304 contiguous bytes of W, then of Y) move between
    // global and shared memory as coalesced 8-byte words; each lane then
    // takes its own row from shared memory (rows 72 bytes apart: no bank
    // conflicts within a half-warp)
    __shared__ float2 rows_s[256 / 32][32 * 9];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int base = (blockIdx.x * (256 / 32) + warp) * 32;
    if (base >= no) return;  // the whole warp
    const int nrow = min(32, no - base);
    float2 *b = rows_s[warp];
    const float2 *src = reinterpret_cast<const float2 *>(W + 18 * (size_t)base);
    for (int k = lane; k < 9 * nrow; k += 32) b[k] = __ldg(src + k);
    __syncwarp();
    float y[18];
    if (lane < nrow) {
        const int o = base + lane;
        const float4 *vi = reinterpret_cast<const float4 *>(Vinv2f + 12 * (size_t)__ldg(obs_pt + o));
        const float4 a = __ldg(vi), bb = __ldg(vi + 1), c = __ldg(vi + 2);
        const float2 s00 = make_float2(a.x, a.y), s01 = make_float2(a.z, a.w), s02 = make_float2(bb.x, bb.y),
                     s11 = make_float2(bb.z, bb.w), s12 = make_float2(c.x, c.y), s22 = make_float2(c.z, c.w);
        float w[18];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const float2 v = b[9 * lane + k];
            w[2 * k] = v.x;
            w[2 * k + 1] = v.y;
        }
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            const float w0 = w[3 * r], w1 = w[3 * r + 1], w2 = w[3 * r + 2];
            y[3 * r + 0] = dot3_df(w0, w1, w2, s00, s01, s02);
            y[3 * r + 1] = dot3_df(w0, w1, w2, s01, s11, s12);
            y[3 * r + 2] = dot3_df(w0, w1, w2, s02, s12, s22);
        }
    }
    __syncwarp();
    if (lane < nrow) {
#pragma unroll
        for (int k = 0; k < 9; ++k) b[9 * lane + k] = make_float2(y[2 * k], y[2 * k + 1]);
    }
    __syncwarp();
    float2 *dst = reinterpret_cast<float2 *>(Y + 18 * (size_t)base);
    for (int k = lane; k < 9 * nrow; k += 32) dst[k] = b[k];
}

// Bulk asynchronous copies between global and shared memory (the copy
// engine of the SM, no registers in flight): a global -> shared copy signals
// an mbarrier with its byte count; a shared -> global copy is a bulk group.
// Addresses and sizes are multiples of 16 bytes.
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ void mbar_init(unsigned long long *bar)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, unsigned long long *bar)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
// waits for phase 0 of the barrier, at most `limit` polls; false if it ran out
__device__ __forceinline__ bool mbar_wait0(unsigned long long *bar, long long limit)
{
    for (long long it = 0; it < limit; ++it) {
        unsigned done;
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0; selp.u32 %0, 1, 0, p; }"
                     : "=r"(done)
                     : "r"(smem_u32(bar))
                     : "memory");
        if (done) return true;
    }
    return false;
}
__device__ __forceinline__ void bulk_s2g(void *dst, const void *src, unsigned bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(smem_u32(src)),
                 "r"(bytes)
                 : "memory");
    asm volatile("cp.async.bulk.commit_group;" ::: "memory");
    asm volatile("cp.async.bulk.wait_group 0;" ::: "memory");
}

// Y = W V^-1 (FP64) for YB_ROWS consecutive observations per CTA: their W
// rows (contiguous, 144 bytes each) come into shared memory by one bulk copy,
// each thread forms its row of Y there (16-byte shared loads at a 144-byte
// stride: no bank conflicts), and one bulk copy writes the CTA's Y rows
// back (the products of compute_Yblks.cl:26-37).  A copy that does not
// complete within poll_limit polls sets status[2] (the trial then reports
// the wait budget exhausted); the CTA then waits for the copy to land in
// its shared memory (at most YB_DRAIN_LIMIT polls: a bulk copy of 37 KB from
// this GPU's own memory completes in microseconds) before it leaves.  Should
// the drain wait also run out, the CTA leaves with the copy possibly still
// in flight; that needs a copy stalled for the whole drain budget, which no
// test provokes.
constexpr int YB_ROWS = 256;
constexpr long long YB_DRAIN_LIMIT = 1LL << 22;

__global__ void __launch_bounds__(YB_ROWS) k_yblocks_bulk(int no, const int *__restrict__ obs_pt,
                                                          const double *__restrict__ W,
                                                          const double *__restrict__ Vinv, double *__restrict__ Y,
                                                          int *__restrict__ status, long long poll_limit)
{
    extern __shared__ __align__(16) double yb_sm[];  // W rows, then Y rows
    __shared__ __align__(8) unsigned long long bar;
    double *sw = yb_sm, *sy = yb_sm + YB_ROWS * 18;
    const int o0 = blockIdx.x * YB_ROWS, rows = min(YB_ROWS, no - o0), t = threadIdx.x;
    const unsigned bytes = (unsigned)rows * 18u * 8u;
    if (t == 0) mbar_init(&bar);
    __syncthreads();
    if (t == 0) bulk_g2s(sw, W + 18 * (size_t)o0, bytes, &bar);
    double s00 = 0, s01 = 0, s02 = 0, s11 = 0, s12 = 0, s22 = 0;
    if (t < rows) {  // the point's V^-1 while the rows arrive
        const double *vi = Vinv + 6 * (size_t)__ldg(obs_pt + o0 + t);
        s00 = __ldg(vi); s01 = __ldg(vi + 1); s02 = __ldg(vi + 2);
        s11 = __ldg(vi + 3); s12 = __ldg(vi + 4); s22 = __ldg(vi + 5);
    }
    if (!mbar_wait0(&bar, poll_limit)) {
        if (t == 0) atomicExch(status + 2, 2);
        mbar_wait0(&bar, YB_DRAIN_LIMIT);  // the copy may still land in this CTA's memory
        return;
    }
    if (t < rows) {
        const double2 *w2 = reinterpret_cast<const double2 *>(sw + 18 * t);
        double w[18], y[18];
#pragma unroll
        for (int e = 0; e < 9; ++e) {
            const double2 v = w2[e];
            w[2 * e] = v.x;
            w[2 * e + 1] = v.y;
        }
#pragma unroll
        for (int r = 0; r < 6; ++r) {
            const double w0 = w[3 * r], w1 = w[3 * r + 1], w2v = w[3 * r + 2];
            y[3 * r + 0] = w0 * s00 + w1 * s01 + w2v * s02;
            y[3 * r + 1] = w0 * s01 + w1 * s11 + w2v * s12;
            y[3 * r + 2] = w0 * s02 + w1 * s12 + w2v * s22;
        }
        double2 *y2 = reinterpret_cast<double2 *>(sy + 18 * t);
#pragma unroll
        for (int e = 0; e < 9; ++e) y2[e] = make_double2(y[2 * e], y[2 * e + 1]);
    }
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // the rows, visible to the bulk copy
    __syncthreads();
    if (t == 0) bulk_s2g(Y + 18 * (size_t)o0, sy, bytes);
}

// The bulk Y kernel's dynamic shared memory (73,728 B) is above the default
// 48 KB limit; the opt-in is a per-device attribute, so it is set once for
// every device a handle is created on, with that device current.
int prepare_device_kernels()
{
    static std::mutex mu;
    static bool done[MAX_DEVICES] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e)), PSBA_ERR_CUDA;
    if (dev < 0 || dev >= MAX_DEVICES) return set_error("device index out of range"), PSBA_ERR_ARG;
    std::lock_guard<std::mutex> lk(mu);
    if (done[dev]) return PSBA_OK;
    e = cudaFuncSetAttribute(k_yblocks_bulk, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)(2 * YB_ROWS * 18 * sizeof(double)));
    if (e != cudaSuccess)
        return set_error(std::string("cudaFuncSetAttribute: ") + cudaGetErrorString(e)), PSBA_ERR_CUDA;
    done[dev] = true;
    return PSBA_OK;
}

void launch_yblocks(const DeviceProblem &d, cudaStream_t s)
{
    if (d.cnp != 6) return launch_yblocks_v(d, s);
    if (d.no == 0) return;
    if (d.prec == PSBA_PREC_FP64) {
        const int smem = (int)(2 * YB_ROWS * 18 * sizeof(double));
        k_yblocks_bulk<<<ceil_div(d.no, YB_ROWS), YB_ROWS, smem, s>>>(d.no, d.obs_pt, d.W, d.Vinv, d.Y, d.status,
                                                                      d.wait_limit);
    } else
        k_yblocks<<<ceil_div(d.no, 256), 256, 0, s>>>(d.no, d.obs_pt, (const float *)d.W, d.Vinv2f, (float *)d.Y);
    note_launch(1);
}

// ---------------------------------------------------------------------------
// Schur complement S = U + mu I - sum_i Y_ik W_il^T (compute_S.cl:39-77) and
// ea = ga - sum_i Y_ij gb_i (compute_ea.cl:21-36).
// Off-diagonal blocks (k > l), all 36 entries of each 6x6 product, into
// partial slots.  Diagonal blocks: one CTA per unit of a camera's
// observations, the 21 lower entries plus the 6 ea sums.  The slots are then
// summed in order (k_schur_reduce).
//
// FP64 products (6-parameter cameras): the pair list cut into equal chunks,
// one per thread of one resident wave, so that every SM issues the same
// number of FP64 multiply-adds; a thread writes its sums to the next slot
// whenever its chunk passes into the next pair.
template <typename R>
__device__ __forceinline__ void off_products(const R *y, const R *w, R *acc)
{
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c < 6; ++c) {
            R s = acc[r * 6 + c];
            s = fma(y[3 * r], w[3 * c], s);
            s = fma(y[3 * r + 1], w[3 * c + 1], s);
            s = fma(y[3 * r + 2], w[3 * c + 2], s);
            acc[r * 6 + c] = s;
        }
}

template <typename R>
__device__ __forceinline__ void schur_off_chunk(int uid, int n_chunks, const SchurUnit *__restrict__ chunks,
                                                const int *__restrict__ pair_start, const int *__restrict__ pa,
                                                const int *__restrict__ pb, const R *__restrict__ Y,
                                                const R *__restrict__ W, double *__restrict__ partial)
{
    if (uid >= n_chunks) return;
    const SchurUnit u = chunks[uid];
    int q = u.slot, slot = u.out;
    int next = __ldg(pair_start + q + 1);  // first entry of the next pair
    const int end = u.begin + u.count;
    double acc[36];
#pragma unroll
    for (int e = 0; e < 36; ++e) acc[e] = 0.0;
    static_assert(is_fp64<R>(), "FP64 products; FP32 products take the unit kernel");
    for (int t = u.begin; t < end; ++t) {
        if (t == next) {
            double *p = partial + (size_t)slot * 36;
#pragma unroll
            for (int e = 0; e < 36; ++e) {
                p[e] = acc[e];
                acc[e] = 0.0;
            }
            ++slot;
            ++q;
            next = __ldg(pair_start + q + 1);
        }
        const int a = __ldg(pa + t), b = __ldg(pb + t);
        R w[18], y[18];
        ldn<R, 18>(W + 18 * (size_t)b, w);
        ldn<R, 18>(Y + 18 * (size_t)a, y);
        off_products<R>(y, w, acc);
    }
    double *p = partial + (size_t)slot * 36;
#pragma unroll
    for (int e = 0; e < 36; ++e) p[e] = acc[e];
}


constexpr int DIAG_NV = 27;  // 21 lower entries + 6 ea sums

// The 21 lower entries of Y W^T into acc (R); the 6 sums of Y gb into eacc
// in FP64 from the exact products in both forms: ea = ga - sum Y gb cancels
// near the optimum, where the step is set by it.
template <typename R>
__device__ __forceinline__ void diag_products(const R *y, const R *w, double g0, double g1, double g2, R *acc,
                                              double *eacc)
{
    int v = 0;
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c, ++v) {
            R s = acc[v];
            s = fma(y[3 * r], w[3 * c], s);
            s = fma(y[3 * r + 1], w[3 * c + 1], s);
            s = fma(y[3 * r + 2], w[3 * c + 2], s);
            acc[v] = s;
        }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        double s = eacc[r];
        s = fma((double)y[3 * r], g0, s);
        s = fma((double)y[3 * r + 1], g1, s);
        s = fma((double)y[3 * r + 2], g2, s);
        eacc[r] = s;
    }
}

// The mixed form's diagonal products: the 21 block sums and the 6 ea sums
// (y . gb) of one observation, all in FP32.
__device__ __forceinline__ void diag_products_f32(const float *y, const float *w, float g0, float g1, float g2,
                                                  float *acc)
{
    int v = 0;
#pragma unroll
    for (int r = 0; r < 6; ++r)
#pragma unroll
        for (int c = 0; c <= r; ++c, ++v) {
            float s = acc[v];
            s = fmaf(y[3 * r], w[3 * c], s);
            s = fmaf(y[3 * r + 1], w[3 * c + 1], s);
            s = fmaf(y[3 * r + 2], w[3 * c + 2], s);
            acc[v] = s;
        }
#pragma unroll
    for (int r = 0; r < 6; ++r) {
        float s = acc[21 + r];
        s = fmaf(y[3 * r], g0, s);
        s = fmaf(y[3 * r + 1], g1, s);
        s = fmaf(y[3 * r + 2], g2, s);
        acc[21 + r] = s;
    }
}

// Diagonal blocks U_k - sum Y W^T (lower 21) and the ea sums (6): one CTA of
// SD_THREADS per unit of <= DIAG_SUPER observations of one camera, SD_PER
// consecutive observations per thread (FP64: accumulated directly; mixed:
// FP32 products over the thread's observations, then one FP64 addition).
// The CTA then sums its threads' partials in a fixed order (each output by
// four threads over 32 partials each, then the four) and writes one partial
// per unit, so a camera has only a handful for k_schur_reduce.  In the mixed
// form the unit's observation and point indices are first gathered into
// shared memory (sidx, 2 DIAG_SUPER ints) by the whole CTA, so a thread's
// walk waits for one L2 round trip per observation instead of three.
// The mixed form's CTA reduction is narrower (two xor-shuffle levels first,
// then 32 partials per output in shared memory): its shared buffer is also
// the off-diagonal warps' index buffer, and a smaller one leaves the L1 more
// room for the rows those warps gather.
constexpr int SD_RED_MX = SD_THREADS / 4;

template <typename R>
__device__ __forceinline__ void schur_diag_cta(const SchurUnit u, const int *__restrict__ cam_obs,
                                               const int *__restrict__ obs_pt, const R *__restrict__ Y,
                                               const R *__restrict__ W, const R *__restrict__ gb,
                                               double *__restrict__ partial, double *red_buf,
                                               int *sidx = nullptr)
{
    static_assert(SD_THREADS == 128 && DIAG_NV * 4 <= SD_THREADS, "four summing threads per output");
    const int t = threadIdx.x;
    double acc[DIAG_NV];
#pragma unroll
    for (int e = 0; e < DIAG_NV; ++e) acc[e] = 0.0;
    const int o1 = min(u.count, (t + 1) * SD_PER);
    if constexpr (is_fp64<R>()) {
        for (int o = t * SD_PER; o < o1; ++o) {
            const int a = __ldg(cam_obs + u.begin + o);
            const int i = __ldg(obs_pt + a);
            R w[18], y[18];
            ldn<R, 18>(W + 18 * (size_t)a, w);
            ldn<R, 18>(Y + 18 * (size_t)a, y);
            const double g0 = __ldg(gb + 3 * (size_t)i), g1 = __ldg(gb + 3 * (size_t)i + 1),
                         g2 = __ldg(gb + 3 * (size_t)i + 2);
            diag_products<R>(y, w, g0, g1, g2, acc, acc + 21);
        }
    } else {
        static_assert(SD_PER <= FLUSH, "one FP32 flush per thread");
        for (int k = t; k < u.count; k += SD_THREADS) {
            const int a = __ldg(cam_obs + u.begin + k);
            sidx[k] = a;
            sidx[DIAG_SUPER + k] = __ldg(obs_pt + a);
        }
        __syncthreads();
        // the block and the ea sums alike: FP32 products summed over the
        // thread's observations (gb rounded to FP32 once per point), then FP64
        float part[DIAG_NV];
#pragma unroll
        for (int e = 0; e < DIAG_NV; ++e) part[e] = 0.0f;
#pragma unroll 2
        for (int o = t * SD_PER; o < o1; ++o) {
            const int a = sidx[o];
            const int i = sidx[DIAG_SUPER + o];
            float w[18], y[18];
            ldn<float, 18>(W + 18 * (size_t)a, w);
            ldn<float, 18>(Y + 18 * (size_t)a, y);
            const float g0 = __ldg(gb + 3 * (size_t)i), g1 = __ldg(gb + 3 * (size_t)i + 1),
                        g2 = __ldg(gb + 3 * (size_t)i + 2);
            diag_products_f32(y, w, g0, g1, g2, part);
        }
        __syncthreads();  // the walk's indices are read: red may overlay them
#pragma unroll
        for (int e = 0; e < DIAG_NV; ++e) acc[e] = (double)part[e];
    }
    // fixed-order CTA sum: each output by four threads over W partials
    // each, then the four (W = 32: one per thread; mixed form, W = 8 per
    // warp after two xor levels over lanes l, l + 8, l + 16, l + 24)
    constexpr int NP = is_fp64<R>() ? SD_THREADS : SD_RED_MX;
    double(*red)[NP + 1] = reinterpret_cast<double(*)[NP + 1]>(red_buf);
    if constexpr (is_fp64<R>()) {
#pragma unroll
        for (int e = 0; e < DIAG_NV; ++e) red[e][t] = acc[e];
    } else {
        const int lane = t & 31;
#pragma unroll
        for (int e = 0; e < DIAG_NV; ++e) {
            double x = acc[e];
            x += __shfl_xor_sync(0xffffffffu, x, 16);
            x += __shfl_xor_sync(0xffffffffu, x, 8);
            if (lane < 8) red[e][(t >> 5) * 8 + lane] = x;
        }
    }
    __syncthreads();
    double s = 0.0;
    const int v = t >> 2, g = t & 3;
    if (v < DIAG_NV) {
#pragma unroll 8
        for (int q = 0; q < NP / 4; ++q) s += red[v][g * (NP / 4) + q];
    }
    __syncthreads();
    if (v < DIAG_NV) red[v][g] = s;
    __syncthreads();
    if (t < DIAG_NV) partial[(size_t)u.out * DIAG_NV + t] = (red[t][0] + red[t][1]) + (red[t][2] + red[t][3]);
}


// FP64 products, 6-parameter cameras: the off-diagonal chunks (blocks below
// off_ctas, 128 threads each) and the diagonal units (the rest) in one
// launch.  Blocks are handed out in index order, so the off-diagonal chunks
// fill one resident wave and the diagonal units run in its tail.
__global__ void __launch_bounds__(128) k_schur(int n_chunks, int off_ctas, const SchurUnit *__restrict__ chunks,
                                               const int *__restrict__ pair_start, const int *__restrict__ pa,
                                               const int *__restrict__ pb, const SchurUnit *__restrict__ diag_units,
                                               const int *__restrict__ cam_obs, const int *__restrict__ obs_pt,
                                               const double *__restrict__ Y, const double *__restrict__ W,
                                               const double *__restrict__ gb, double *__restrict__ off_partial,
                                               double *__restrict__ diag_partial)
{
    static_assert(SD_THREADS == 128, "one block size for both parts");
    __shared__ double red[DIAG_NV][SD_THREADS + 1];
    if ((int)blockIdx.x < off_ctas)
        schur_off_chunk<double>(blockIdx.x * 128 + threadIdx.x, n_chunks, chunks, pair_start, pa, pb, Y, W,
                                off_partial);
    else
        schur_diag_cta<double>(diag_units[blockIdx.x - off_ctas], cam_obs, obs_pt, Y, W, gb, diag_partial, &red[0][0]);
}

int schur_off_wave_threads()
{
    // one resident wave of k_schur, per device (the serving lanes' threads
    // ask at the same time)
    static std::mutex mu;
    static int threads[MAX_DEVICES] = {};
    int dev = 0;
    cudaGetDevice(&dev);
    if (dev < 0 || dev >= MAX_DEVICES) dev = 0;
    std::lock_guard<std::mutex> lk(mu);
    if (threads[dev] == 0) {
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_schur, 128, 0);
        threads[dev] = std::max(1, sms) * std::max(1, per_sm) * 128;
    }
    return threads[dev];
}

// FP32 products, 6-parameter cameras: one warp per unit of <= MX_UNIT
// entries of one camera pair.  The warp first copies the unit's two index
// lists into shared memory (coalesced), so that each step waits for one L2
// round trip (the rows) instead of two.  Lane 4 s + q then works on the
// entries s, s + 8, s + 16, ... of the unit (s = 0..7) and on quadrant q of
// the 6 x 6 block (rows 3 (q >> 1) .. +2, columns 3 (q & 1) .. +2): it loads
// the nine Y values of its rows and the nine W values of its columns (the
// four lanes of an entry read two 36-byte halves of each row, so the
// requests of a warp instruction are eight rows' worth) and keeps nine FP32
// sums, in two interleaved sets (entries s, s + 16, ... and s + 8, s + 24,
// ...: two independent chains of at most 16 products each, added in FP32 at
// the end, so a lane's sum covers at most 32 products).  The eight entry
// slots are combined in FP64 by a fixed xor tree and the unit's partial goes
// to its slot; k_schur_reduce sums a pair's units in order, in FP64.  Every
// sum has a fixed order, so the result does not depend on scheduling.
// Nine consecutive floats of a row half: the half starts at float 9 h of a
// 72-byte row (row start 8-byte aligned), so it is one scalar and four
// 8-byte pairs -- the scalar last for h = 0, first for h = 1 -- five loads
// instead of nine (the L1 is what bounds this kernel).
__device__ __forceinline__ void ld_half(const float *__restrict__ row, int h, float (&v)[9])
{
    const float *p = row + 9 * h;
    const float single = __ldg(p + (h ? 0 : 8));
    const float2 *q = reinterpret_cast<const float2 *>(p + (h ? 1 : 0));
    float pr[8];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const float2 t = __ldg(q + k);
        pr[2 * k] = t.x;
        pr[2 * k + 1] = t.y;
    }
    v[0] = h ? single : pr[0];
#pragma unroll
    for (int e = 1; e < 8; ++e) v[e] = h ? pr[e - 1] : pr[e];
    v[8] = h ? pr[7] : single;
}

__device__ __forceinline__ void mx_quadrant(const float *__restrict__ Y, const float *__restrict__ W, int a, int b,
                                            int qr, int qc, float *acc)
{
    float y[9], w[9];
    ld_half(Y + 18 * (size_t)a, qr, y);
    ld_half(W + 18 * (size_t)b, qc, w);
#pragma unroll
    for (int i = 0; i < 3; ++i)
#pragma unroll
        for (int j = 0; j < 3; ++j) {
            float s = acc[3 * i + j];
            s = fmaf(y[3 * i], w[3 * j], s);
            s = fmaf(y[3 * i + 1], w[3 * j + 1], s);
            s = fmaf(y[3 * i + 2], w[3 * j + 2], s);
            acc[3 * i + j] = s;
        }
}

// The rows of one step (sixteen entries: their Y rows and W rows, 288
// float pairs) are loaded by the whole warp, each lane the same nine
// (row, pair) slots at every step, and meet the lanes that use them in
// shared memory: a warp load instruction then covers ~256 contiguous bytes
// of about four rows instead of fifteen sectors of eight, which cuts the L1
// wavefronts the gathers cost (the kernel's bound).  The next step's pairs
// are loaded into registers while the current one is summed.  Lane 4s + q
// sums entry s of the step into a0 and entry s + 8 into a1 (the order of the
// per-entry loads it replaced).
constexpr int MX_STEP = 16;                 // entries per step
constexpr int MX_PAIRS = 2 * MX_STEP * 9;   // float pairs of one step's rows
constexpr int MX_ROWF = 2 * MX_PAIRS;       // their floats in shared memory
constexpr int MX_SLOTS = MX_PAIRS / 32 + (MX_PAIRS % 32 != 0);  // pairs a lane loads per step

__device__ __forceinline__ void schur_off_warp(const SchurUnit u, const int *__restrict__ pa,
                                               const int *__restrict__ pb, const float *__restrict__ Y,
                                               const float *__restrict__ W, int *sidx, float *rowf,
                                               double *__restrict__ partial)
{
    const int lane = threadIdx.x & 31, s = lane >> 2, q = lane & 3, qr = q >> 1, qc = q & 1;
    int *ia = sidx, *ib = sidx + MX_UNIT;
    for (int t = lane; t < u.count; t += 32) {
        ia[t] = __ldg(pa + u.begin + t);
        ib[t] = __ldg(pb + u.begin + t);
    }
    __syncwarp();
    // this lane's slots: pair k = lane + 32 m of the step's; row r = k / 9
    // (0-15: Y of entry r, 16-31: W of entry r - 16), pair k % 9 of the row
    auto load_step = [&](int t0, float2 (&v)[MX_SLOTS]) {
#pragma unroll
        for (int m = 0; m < MX_SLOTS; ++m) {
            const int kk = lane + 32 * m, r = kk / 9, t = t0 + (r & (MX_STEP - 1));
            if (kk < MX_PAIRS && t < u.count) {
                const float *row = r < MX_STEP ? Y + 18 * (size_t)ia[t] : W + 18 * (size_t)ib[t];
                v[m] = __ldg(reinterpret_cast<const float2 *>(row) + (kk - 9 * r));
            }
        }
    };
    float a0[9], a1[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) a0[e] = a1[e] = 0.0f;
    auto prod = [&](const float *yrow, const float *wrow, float (&acc)[9]) {
        float y[9], w[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) {
            y[e] = yrow[e];
            w[e] = wrow[e];
        }
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) {
                float sm = acc[3 * i + j];
                sm = fmaf(y[3 * i], w[3 * j], sm);
                sm = fmaf(y[3 * i + 1], w[3 * j + 1], sm);
                sm = fmaf(y[3 * i + 2], w[3 * j + 2], sm);
                acc[3 * i + j] = sm;
            }
    };
    float2 nxt[MX_SLOTS];
    load_step(0, nxt);
    for (int t0 = 0; t0 < u.count; t0 += MX_STEP) {
        __syncwarp();  // the previous step's rows are read
#pragma unroll
        for (int m = 0; m < MX_SLOTS; ++m)
            if (lane + 32 * m < MX_PAIRS) reinterpret_cast<float2 *>(rowf)[lane + 32 * m] = nxt[m];
        __syncwarp();
        if (t0 + MX_STEP < u.count) load_step(t0 + MX_STEP, nxt);
        if (t0 + s < u.count)
            prod(rowf + 18 * s + 9 * qr, rowf + 18 * (MX_STEP + s) + 9 * qc, a0);
        if (t0 + 8 + s < u.count)
            prod(rowf + 18 * (8 + s) + 9 * qr, rowf + 18 * (MX_STEP + 8 + s) + 9 * qc, a1);
    }
    double v[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) {
        double x = (double)(a0[e] + a1[e]);
        x += __shfl_xor_sync(0xffffffffu, x, 4);
        x += __shfl_xor_sync(0xffffffffu, x, 8);
        x += __shfl_xor_sync(0xffffffffu, x, 16);
        v[e] = x;
    }
    if (s == 0) {
        double *p = partial + (size_t)u.out * 36 + 18 * qr + 3 * qc;
#pragma unroll
        for (int i = 0; i < 3; ++i)
#pragma unroll
            for (int j = 0; j < 3; ++j) p[6 * i + j] = v[3 * i + j];
    }
}

// FP32 products: the diagonal units first (one CTA each, blocks below
// n_diag: they walk their observations one after another, so they start
// early and run beside the off-diagonal units), then the off-diagonal units
// (four per block, a warp each).
#ifndef PSBA_SF32_MINB
#define PSBA_SF32_MINB 6  // blocks per SM that k_schur_f32's register budget aims at (tuning knob)
#endif
__global__ void __launch_bounds__(128, PSBA_SF32_MINB) k_schur_f32(int n_units, int n_diag, const SchurUnit *__restrict__ units,
                                                   const int *__restrict__ pa, const int *__restrict__ pb,
                                                   const SchurUnit *__restrict__ diag_units,
                                                   const int *__restrict__ cam_obs, const int *__restrict__ obs_pt,
                                                   const float *__restrict__ Y, const float *__restrict__ W,
                                                   const float *__restrict__ gb32, double *__restrict__ off_partial,
                                                   double *__restrict__ diag_partial)
{
    // one shared buffer: a diagonal unit's indices, then its reduction
    // (after a barrier), or the four warps' index lists
    constexpr int RED_WORDS = DIAG_NV * (SD_RED_MX + 1) * 2, IDX_WORDS = 4 * 2 * MX_UNIT;
    constexpr int OFF_WORDS = IDX_WORDS + 4 * MX_ROWF;  // + each warp's step rows
    static_assert(IDX_WORDS >= 2 * DIAG_SUPER, "the index buffer holds a diagonal unit's indices");
    __shared__ __align__(16) int buf[RED_WORDS > OFF_WORDS ? RED_WORDS : OFF_WORDS];
    if ((int)blockIdx.x < n_diag) {
        schur_diag_cta<float>(diag_units[blockIdx.x], cam_obs, obs_pt, Y, W, gb32, diag_partial,
                              reinterpret_cast<double *>(buf), buf);
    } else {
        const int uid = (blockIdx.x - n_diag) * 4 + (threadIdx.x >> 5);
        if (uid < n_units) schur_off_warp(units[uid], pa, pb, Y, W, buf + (threadIdx.x >> 5) * 2 * MX_UNIT,
                                          reinterpret_cast<float *>(buf + IDX_WORDS) + (threadIdx.x >> 5) * MX_ROWF,
                                          off_partial);
    }
}

// Sum unit partials into S (lower) and rhs = ea.
__global__ void k_schur_reduce(int n_pairs, int nc, int Np, const int *__restrict__ pair_kl,
                               const int *__restrict__ off_start, const double *__restrict__ off_partial,
                               const int *__restrict__ diag_start,
                               const double *__restrict__ diag_partial,
                               const double *__restrict__ U, const double *__restrict__ g, double mu,
                               double *__restrict__ S, double *__restrict__ rhs)
{
    const int id = blockIdx.x * blockDim.x + threadIdx.x;
    const int n_off = n_pairs * 36;
    if (id < n_off) {
        const int p = id / 36, v = id % 36;
        double sum = 0.0;
        for (int u = off_start[p]; u < off_start[p + 1]; ++u) sum += off_partial[(size_t)u * 36 + v];
        const int k = pair_kl[2 * p], l = pair_kl[2 * p + 1];
        const int r = v / 6, c = v % 6;
        S[(size_t)(6 * k + r) * Np + 6 * l + c] = -sum;
        return;
    }
    const int id2 = id - n_off;
    if (id2 >= nc * DIAG_NV) return;
    const int k = id2 / DIAG_NV, v = id2 % DIAG_NV;
    double sum = 0.0;
    for (int u = diag_start[k]; u < diag_start[k + 1]; ++u) sum += diag_partial[(size_t)u * DIAG_NV + v];
    if (v >= 21) {
        const int r = v - 21;
        rhs[6 * k + r] = g[6 * k + r] - sum;
        return;
    }
    int r = 0, c = 0, kk = v;
    for (r = 0; r < 6; ++r) {
        if (kk <= r) {
            c = kk;
            break;
        }
        kk -= r + 1;
    }
    const double uu = U[36 * (size_t)k + r * 6 + c];
    S[(size_t)(6 * k + r) * Np + 6 * k + c] = (r == c ? uu + mu : uu) - sum;
}

__global__ void k_pad_identity(int N, int Np, double *S, double *rhs)
{
    const int i = N + blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Np) return;
    S[(size_t)i * Np + i] = 1.0;
    rhs[i] = 0.0;
}

void launch_schur_off(const DeviceProblem &d, cudaStream_t s)
{
    if (d.cnp != 6) return launch_schur_off_v(d, s);
    if (d.prec == PSBA_PREC_FP64) {
        // the diagonal units ride in the same launch (k_schur)
        const int off_ctas = ceil_div(d.n_off_chunks, 128);
        if (off_ctas + d.n_diag_units == 0) return;
        k_schur<<<off_ctas + d.n_diag_units, 128, 0, s>>>(
            d.n_off_chunks, off_ctas, d.off_chunks, d.pair_start, d.pair_a, d.pair_b, d.diag_units, d.cam_obs,
            d.obs_pt, d.Y, d.W, d.g + d.N, d.schur_partial, d.schur_partial + off_partial_slots(d) * 36);
        note_launch(1);
        return;
    }
    const int off_ctas = ceil_div(d.n_mx_units, 4);
    if (off_ctas + d.n_diag_units == 0) return;
    k_schur_f32<<<off_ctas + d.n_diag_units, 128, 0, s>>>(
        d.n_mx_units, d.n_diag_units, d.mx_units, d.pair_a, d.pair_b, d.diag_units, d.cam_obs, d.obs_pt,
        (const float *)d.Y, (const float *)d.W, d.gb32, d.schur_partial,
        d.schur_partial + off_partial_slots(d) * 36);
    note_launch(1);
}

void launch_schur_diag(const DeviceProblem &d, cudaStream_t s)
{
    // 6-parameter cameras: the diagonal units run in the off-diagonal launch
    // (k_schur, k_schur_f32)
    if (d.cnp != 6) launch_schur_diag_v(d, s);
}

void launch_schur_reduce(const DeviceProblem &d, double mu, cudaStream_t s)
{
    cudaMemsetAsync(d.S, 0, sizeof(double) * (size_t)d.Np * d.Np, s);
    if (d.cnp != 6) {
        launch_schur_reduce_v(d, mu, s);
        if (d.Np > d.N) {
            k_pad_identity<<<1, TILE, 0, s>>>(d.N, d.Np, d.S, d.rhs);
            note_launch(1);
        }
        return;
    }
    double *off_partial = d.schur_partial;
    double *diag_partial = d.schur_partial + off_partial_slots(d) * 36;
    const int total = d.n_pairs * 36 + d.nc * DIAG_NV;
    const int *off_start = d.prec == PSBA_PREC_FP64 ? d.off_chunk_start : d.mx_unit_start;
    k_schur_reduce<<<ceil_div(total, 128), 128, 0, s>>>(d.n_pairs, d.nc, d.Np, d.pair_kl,
                                                          off_start, off_partial,
                                                          d.diag_unit_start, diag_partial, d.U, d.g,
                                                          mu, d.S, d.rhs);
    note_launch(1);
    if (d.Np > d.N) {
        k_pad_identity<<<1, TILE, 0, s>>>(d.N, d.Np, d.S, d.rhs);
        note_launch(1);
    }
}

void launch_schur(const DeviceProblem &d, double mu, cudaStream_t s)
{
    launch_schur_off(d, s);
    launch_schur_diag(d, s);
    launch_schur_reduce(d, mu, s);
}

// dp_L2 = |dp|^2 and rho_den = dp (mu dp + g) from the camera part of dp and
// the per-block sums of the point part, in a fixed order; the Cholesky
// status.  One block of 256 threads.
__device__ void finish_trial_block(int ncp, int nblocks, const double *__restrict__ dp,
                                   const double *__restrict__ g, double mu, const double *partial,
                                   const int *__restrict__ status, TrialScalars *__restrict__ out)
{
    __shared__ double r0[256], r1[256];
    double a = 0.0, b = 0.0;
    for (int k = threadIdx.x; k < ncp; k += 256) {
        const double x = __ldcg(dp + k);
        a += x * x;
        b += x * (mu * x + g[k]);
    }
    for (int k = threadIdx.x; k < nblocks; k += 256) {
        a += __ldcg(partial + 2 * k);
        b += __ldcg(partial + 2 * k + 1);
    }
    r0[threadIdx.x] = a;
    r1[threadIdx.x] = b;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) {
            r0[threadIdx.x] += r0[threadIdx.x + st];
            r1[threadIdx.x] += r1[threadIdx.x + st];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out->dp_L2 = r0[0];
        out->rho_den = r1[0];
        out->chol_status = status[0] != 0 ? status[0] : (status[2] != 0 ? 2 : 0);  // [2]: a bulk copy's wait
    }
}

// ---------------------------------------------------------------------------
// eb = gb - sum_j W_ij^T dpa_j (compute_eb.cl:25-39), dpb = V^-1 eb
// (compute_dpb.cl:19-34); block partials of |dpb|^2 and dpb (mu dpb + gb)
// for the gain ratio (levmar.cpp:271-280).  The sums over a point's
// observations take 3 m lanes, m = 1..4 by its views (points in pt_order,
// up to ten a warp, eight warps a block, per the eb_warps schedule), so no
// lane walks more than ~10 observations; the rest of a point takes one
// thread, so its FP64 instructions issue with most lanes busy.
template <typename R>
__global__ void __launch_bounds__(256) k_eb_dpb(int np, int ncp, const int2 *__restrict__ eb_warps,
                                                const int *__restrict__ pt_start,
                                                const int *__restrict__ pt_order,
                                                const int *__restrict__ obs_cam,
                                                const R *__restrict__ W, const double *__restrict__ Vinv,
                                                const double *__restrict__ g, double mu,
                                                double *__restrict__ dp, double *__restrict__ eb,
                                                double *__restrict__ partial, int stage,
                                                const int *__restrict__ status, int *__restrict__ ticket,
                                                TrialScalars *__restrict__ out, const float2 *__restrict__ dpa2f,
                                                const double *__restrict__ pts, float2 *__restrict__ x2f)
{
    static_assert(EB_WARPS == 8, "eight warps a block");
    __shared__ double s_sum[EB_PPB][3];
    __shared__ double r0[EB_WARPS], r1[EB_WARPS];
    extern __shared__ double s_dpa[];  // the camera part of dp (ncp doubles) when staged
    // the mixed form, staged: dpa as FP32 pairs (hi, lo), the products in
    // double-float arithmetic, so no FP64 instruction per observation
    constexpr bool DF = !is_fp64<R>();
    float2 *s_dpa2 = reinterpret_cast<float2 *>(s_dpa);
    if (stage) {
        if (DF && dpa2f)
            for (int e = threadIdx.x; e < ncp; e += blockDim.x) s_dpa2[e] = dpa2f[e];
        else
            for (int e = threadIdx.x; e < ncp; e += blockDim.x) s_dpa[e] = dp[e];
        __syncthreads();
    }
    const double *dpa = stage ? s_dpa : dp;
    const bool df = DF && stage && dpa2f;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int first = eb_warps[blockIdx.x * EB_WARPS].x;  // the block's points: [first, last) in pt_order
    const int last = eb_warps[(blockIdx.x + 1) * EB_WARPS].x;
    // the warp's points: 3 m lanes each; lane (s, c) sums component c of
    // W^T dpa over the observations s, s + m, s + 2m, ... of its point
    {
        const int2 wi = eb_warps[blockIdx.x * EB_WARPS + warp];
        const int npw = eb_warps[blockIdx.x * EB_WARPS + warp + 1].x - wi.x, m = wi.y;
        const int lpp = 3 * m, pw = lane / lpp, r = lane - lpp * pw, s = r / 3, c = r - 3 * s;
        double part = 0.0;
        if (df) {
            // two double-float accumulators (hi, lo): w dpa_hi split exactly
            // by an FMA, the sum carried by TwoSum, w dpa_lo and the errors
            // summed in lo; converted to FP64 once per lane
            float h0 = 0.0f, l0 = 0.0f, h1 = 0.0f, l1 = 0.0f;
            if (pw < npw) {
                const int i = pt_order[wi.x + pw];
                const int end = pt_start[i + 1];
#pragma unroll 2
                for (int o = pt_start[i] + s; o < end; o += m) {
                    const float *w = reinterpret_cast<const float *>(W) + 18 * (size_t)o;
                    const float2 *da = s_dpa2 + 6 * (size_t)__ldg(obs_cam + o);
#pragma unroll
                    for (int k = 0; k < 6; ++k) {
                        const float wv = w[3 * k + c];
                        const float2 d2 = da[k];
                        const float p = __fmul_rn(wv, d2.x);
                        const float pe = fmaf(wv, d2.x, -p);
                        float t;
                        if (k & 1) {
                            two_sum_f(h1, p, h1, t);
                            l1 = fmaf(wv, d2.y, l1 + (t + pe));
                        } else {
                            two_sum_f(h0, p, h0, t);
                            l0 = fmaf(wv, d2.y, l0 + (t + pe));
                        }
                    }
                }
            }
            // the two accumulators and then the m lanes of a component
            // meet in double-float as well (in order of s), converted once
            // (each lane's own partial is what is exchanged, not a running sum)
            float hp, t;
            two_sum_f(h0, h1, hp, t);
            const float lp = (l0 + l1) + t;
            float hs = hp, ls = lp;
#pragma unroll
            for (int q = 1; q < 4; ++q) {
                const int src = min(lpp * pw + 3 * q + c, 31);
                const float oh = __shfl_sync(0xffffffffu, hp, src);
                const float ol = __shfl_sync(0xffffffffu, lp, src);
                if (q < m) {
                    two_sum_f(hs, oh, hs, t);
                    ls += ol + t;
                }
            }
            if (pw < npw && s == 0) s_sum[wi.x + pw - first][c] = (double)hs + (double)ls;
        } else {
            // one accumulator per camera parameter: six short chains
            double acc[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
            if (pw < npw) {
                const int i = pt_order[wi.x + pw];
                const int end = pt_start[i + 1];
#pragma unroll 4
                for (int o = pt_start[i] + s; o < end; o += m) {
                    const R *w = W + 18 * (size_t)o;
                    const double *da = dpa + 6 * (size_t)__ldg(obs_cam + o);
#pragma unroll
                    for (int k = 0; k < 6; ++k) acc[k] = fma((double)w[3 * k + c], da[k], acc[k]);
                }
            }
            part = ((acc[0] + acc[1]) + (acc[2] + acc[3])) + (acc[4] + acc[5]);
            // the m partial sums of a component, in order of s (each lane's
            // own partial is what is exchanged, not a running sum)
            double e = part;
#pragma unroll
            for (int q = 1; q < 4; ++q) {
                const double v = __shfl_sync(0xffffffffu, part, min(lpp * pw + 3 * q + c, 31));
                if (q < m) e += v;
            }
            if (pw < npw && s == 0) s_sum[wi.x + pw - first][c] = e;
        }
    }
    __syncthreads();
    // one thread per point finishes it: eb = gb - W^T dpa, dpb = V^-1 eb
    double s_sq = 0.0, s_rho = 0.0;
    const int t = threadIdx.x;
    const int slot = first + t;
    if (slot < last) {
        const int i = pt_order[slot];
        const double *gb = g + ncp + 3 * (size_t)i;
        const double e0 = gb[0] - s_sum[t][0], e1 = gb[1] - s_sum[t][1], e2 = gb[2] - s_sum[t][2];
        eb[3 * (size_t)i] = e0;
        eb[3 * (size_t)i + 1] = e1;
        eb[3 * (size_t)i + 2] = e2;
        const double *vi = Vinv + 6 * (size_t)i;
        const double v0 = vi[0], v1 = vi[1], v2 = vi[2], v3 = vi[3], v4 = vi[4], v5 = vi[5];
        const double d0 = v0 * e0 + v1 * e1 + v2 * e2;
        const double d1 = v1 * e0 + v3 * e1 + v4 * e2;
        const double d2 = v2 * e0 + v4 * e1 + v5 * e2;
        double *db = dp + ncp + 3 * (size_t)i;
        db[0] = d0;
        db[1] = d1;
        db[2] = d2;
        if (x2f) {  // the mixed trial cost's point, pts + dpb as FP32 pairs
            const double *X = pts + 3 * (size_t)i;
            x2f[3 * (size_t)i] = split2f(X[0] + d0);
            x2f[3 * (size_t)i + 1] = split2f(X[1] + d1);
            x2f[3 * (size_t)i + 2] = split2f(X[2] + d2);
        }
        s_sq = d0 * d0 + d1 * d1 + d2 * d2;
        s_rho = d0 * (mu * d0 + gb[0]) + d1 * (mu * d1 + gb[1]) + d2 * (mu * d2 + gb[2]);
    }
    // block sums in a fixed order: the finishing warps, then the warps' sums
    constexpr int FW = (EB_PPB + 31) / 32;
    if (warp < FW) {
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            s_sq += __shfl_xor_sync(0xffffffffu, s_sq, off);
            s_rho += __shfl_xor_sync(0xffffffffu, s_rho, off);
        }
        if (lane == 0) {
            r0[warp] = s_sq;
            r1[warp] = s_rho;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = r0[0], b = r1[0];
#pragma unroll
        for (int w = 1; w < FW; ++w) {
            a += r0[w];
            b += r1[w];
        }
        partial[2 * blockIdx.x] = a;
        partial[2 * blockIdx.x + 1] = b;
    }
    // the last block adds the camera part and every block's sums (the
    // trial's step scalars)
    if (take_last_ticket(ticket)) {
        finish_trial_block(ncp, gridDim.x, dp, g, mu, partial, status, out);
        if (threadIdx.x == 0) *ticket = 0;
    }
}

// k_eb_dpb blocks: EB_WARPS warps of the schedule each, at least np / EB_PPB
// (the variable-intrinsics version uses one thread per point, and its
// surplus blocks write zero partials)
int eb_blocks(const DeviceProblem &d) { return d.n_eb_warps / EB_WARPS; }

void launch_eb_dpb(const DeviceProblem &d, double mu, cudaStream_t s)
{
    if (d.cnp != 6) return launch_eb_dpb_v(d, mu, eb_blocks(d), s);
    // the camera part of dp in shared memory when it fits: each observation
    // reads its camera's six values
    const int stage = (size_t)d.N * sizeof(double) <= 48 * 1024 ? 1 : 0;
    const size_t smem = stage ? sizeof(double) * d.N : 0;
    if (d.prec == PSBA_PREC_FP64)
        k_eb_dpb<double><<<eb_blocks(d), 256, smem, s>>>(d.np, d.N, d.eb_warps, d.pt_start, d.pt_order, d.obs_cam,
                                                           d.W, d.Vinv, d.g, mu, d.dp, d.eb, d.red_partial, stage,
                                                           d.status, d.tickets, d.scal, nullptr, nullptr, nullptr);
    else
        k_eb_dpb<float><<<eb_blocks(d), 256, smem, s>>>(d.np, d.N, d.eb_warps, d.pt_start, d.pt_order, d.obs_cam,
                                                          (const float *)d.W, d.Vinv, d.g, mu, d.dp, d.eb,
                                                          d.red_partial, stage, d.status, d.tickets, d.scal,
                                                          d.dpa2f, d.pts, d.wt ? nullptr : d.x2f);
    note_launch(1);
}

// Sum the dpa part and the per-block partials of the back-substitution in a
// fixed order; copy the Cholesky status.  One block (11/16-parameter
// cameras; for 6-parameter cameras k_eb_dpb's last block does this).
__global__ void k_finish_trial(int ncp, int nblocks, const double *__restrict__ dp,
                               const double *__restrict__ g, double mu,
                               const double *__restrict__ partial, const int *__restrict__ status,
                               TrialScalars *__restrict__ out)
{
    finish_trial_block(ncp, nblocks, dp, g, mu, partial, status, out);
}

void launch_finish_trial(const DeviceProblem &d, double mu, cudaStream_t s)
{
    if (d.cnp == 6) return;  // k_eb_dpb's last block did it
    k_finish_trial<<<1, 256, 0, s>>>(d.N, eb_blocks(d), d.dp, d.g, mu, d.red_partial, d.status,
                                     d.scal); note_launch(1);
}

// Fixed-order sum of n partials into *dst (one block).
__global__ void k_sum_partials(const double *__restrict__ partial, int n, double *__restrict__ dst)
{
    __shared__ double r[256];
    double a = 0.0;
    for (int k = threadIdx.x; k < n; k += 256) a += partial[k];
    r[threadIdx.x] = a;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) r[threadIdx.x] += r[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) *dst = r[0];
}

void launch_sum_partials(const double *partial, int n, double *dst, cudaStream_t s)
{
    k_sum_partials<<<1, 256, 0, s>>>(partial, n, dst); note_launch(1);
}

// max(0, x[k]) over k (maxElmOfUV starts from 0, sba_func.cpp:433-440), NaN
// ignored as fmax does: per block, then combined with an integer atomicMax
// on the bit patterns, which order like the values for non-negative
// doubles; *dst is zeroed first.  Exact in any order.
__global__ void k_max_uvdiag(const double *__restrict__ x, int n, double *__restrict__ dst)
{
    __shared__ double r[256];
    double m = 0.0;
    for (int k = blockIdx.x * 256 + threadIdx.x; k < n; k += gridDim.x * 256) m = fmax(m, x[k]);
    r[threadIdx.x] = m;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) r[threadIdx.x] = fmax(r[threadIdx.x], r[threadIdx.x + st]);
        __syncthreads();
    }
    if (threadIdx.x == 0 && r[0] > 0.0)
        atomicMax(reinterpret_cast<unsigned long long *>(dst), (unsigned long long)__double_as_longlong(r[0]));
}

void launch_max_uvdiag(const DeviceProblem &d, double *dst, cudaStream_t s)
{
    const int n = d.N + 3 * d.np;
    cudaMemsetAsync(dst, 0, sizeof(double), s);
    k_max_uvdiag<<<std::max(1, std::min(ceil_div(n, 256 * 8), 304)), 256, 0, s>>>(d.uvdiag, n, dst);
    note_launch(1);
}

// Two-pass fixed-order reductions over long vectors.
__global__ void k_sumsq_partial(const double *__restrict__ x, const double *__restrict__ y, long long n,
                                double *__restrict__ partial)
{
    __shared__ double r[256];
    double a = 0.0;
    const long long stride = (long long)gridDim.x * 256;
    for (long long k = (long long)blockIdx.x * 256 + threadIdx.x; k < n; k += stride)
        a += y ? x[k] * y[k] : x[k] * x[k];
    r[threadIdx.x] = a;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) r[threadIdx.x] += r[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = r[0];
}

// The parameters' squared norms for the LM stop test (levmar.cpp:150-152):
// blocks below nred stride over the points' coordinates, block nred over
// the cameras' parameters; fixed-order sums in every block and in the last.
__global__ void __launch_bounds__(256) k_param_norm(const double *__restrict__ cams, int ncv,
                                                    const double *__restrict__ pts, long long npv, int nred,
                                                    double *__restrict__ partial, int *__restrict__ ticket,
                                                    double *__restrict__ dst_cams, double *__restrict__ dst_pts)
{
    __shared__ double r[256];
    double a = 0.0;
    if ((int)blockIdx.x < nred) {
        const long long stride = (long long)nred * 256;
        for (long long k = (long long)blockIdx.x * 256 + threadIdx.x; k < npv; k += stride) a = fma(pts[k], pts[k], a);
    } else {
        for (int k = threadIdx.x; k < ncv; k += 256) a = fma(cams[k], cams[k], a);
    }
    r[threadIdx.x] = a;
    __syncthreads();
    for (int st = 128; st > 0; st >>= 1) {
        if (threadIdx.x < st) r[threadIdx.x] += r[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = r[0];
    if (take_last_ticket(ticket)) {
        sum_partials_block(partial, nred, dst_pts);
        if (threadIdx.x == 0) {
            *dst_cams = __ldcg(partial + nred);
            *ticket = 0;
        }
    }
}

void launch_param_norm(const DeviceProblem &d, int nred, double *partial, double *dst_cams, double *dst_pts,
                       cudaStream_t s)
{
    k_param_norm<<<nred + 1, 256, 0, s>>>(d.cams, d.N, d.pts, 3LL * d.np, nred, partial, d.tickets + 2, dst_cams,
                                          dst_pts);
    note_launch(1);
}

void launch_dot(const double *x, const double *y, long long n, double *partial, int nblocks,
                double *dst, cudaStream_t s)
{
    k_sumsq_partial<<<nblocks, 256, 0, s>>>(x, y, n, partial); note_launch(1);
    k_sum_partials<<<1, 256, 0, s>>>(partial, nblocks, dst); note_launch(1);
}

// Accept a step: cams += dpa, pts += dpb (compute_newp.cl + update_p.cl).
__global__ void k_update_params(int ncp, int npp, double *cams, double *pts, const double *dp)
{
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < ncp)
        cams[k] = cams[k] + dp[k];
    else if (k < ncp + npp)
        pts[k - ncp] = pts[k - ncp] + dp[k];
}

void launch_update_params(const DeviceProblem &d, cudaStream_t s)
{
    const int n = d.N + 3 * d.np;
    k_update_params<<<ceil_div(n, 256), 256, 0, s>>>(d.N, 3 * d.np, d.cams, d.pts, d.dp); note_launch(1);
}

// J x per observation (compute_Jmultiply.cl:28-44), 2 outputs each.
template <typename R>
__global__ void k_jmultiply(int no, int ncp, const int *__restrict__ obs_pt,
                            const int *__restrict__ obs_cam, const R *__restrict__ A,
                            const R *__restrict__ B, const double *__restrict__ x,
                            double *__restrict__ out)
{
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    if (o >= no) return;
    const double *xa = x + 6 * (size_t)obs_cam[o];
    const double *xb = x + ncp + 3 * (size_t)obs_pt[o];
    const R *a = A + 12 * (size_t)o;
    const R *b = B + 6 * (size_t)o;
    for (int k = 0; k < 2; ++k) {
        double s = 0.0;
        for (int m = 0; m < 6; ++m) s += (double)a[6 * k + m] * xa[m];
        for (int m = 0; m < 3; ++m) s += (double)b[3 * k + m] * xb[m];
        out[2 * (size_t)o + k] = s;
    }
}

void launch_jmultiply(const DeviceProblem &d, const double *x, double *out, cudaStream_t s)
{
    if (d.cnp != 6) return launch_jmultiply_v(d, x, out, s);
    if (d.no == 0) return;
    if (d.prec == PSBA_PREC_FP64)
        k_jmultiply<double><<<ceil_div(d.no, 256), 256, 0, s>>>(d.no, d.N, d.obs_pt, d.obs_cam, d.A, d.B, x, out);
    else
        k_jmultiply<float><<<ceil_div(d.no, 256), 256, 0, s>>>(d.no, d.N, d.obs_pt, d.obs_cam,
                                                                 (const float *)d.A, (const float *)d.B, x, out);
    note_launch(1);
}

__global__ void k_axpby(double *out, const double *x, double a, const double *y, double b, long long n)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = y ? a * x[k] + b * y[k] : a * x[k];
}

void launch_axpby(double *out, const double *x, double a, const double *y, double b, long long n,
                  cudaStream_t s)
{
    k_axpby<<<ceil_div(n, 256), 256, 0, s>>>(out, x, a, y, b, n); note_launch(1);
}

// out = sign * (x * num) / (den_scale * den) with num, den on the device.
__global__ void k_scale(double *out, const double *x, const double *num, const double *den,
                        double den_scale, double sign, long long n)
{
    const long long k = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) out[k] = sign * (x[k] * (*num)) / (den_scale * (*den));
}

void launch_scale(double *out, const double *x, const double *num, const double *den,
                  double den_scale, double sign, long long n, cudaStream_t s)
{
    k_scale<<<ceil_div(n, 256), 256, 0, s>>>(out, x, num, den, den_scale, sign, n); note_launch(1);
}

template <typename R>
__global__ void k_expand_V(int np, const R *V6, double *V9)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= np) return;
    const R *v = V6 + 6 * (size_t)i;
    double *o = V9 + 9 * (size_t)i;
    o[0] = v[0]; o[1] = v[1]; o[2] = v[2];
    o[3] = v[1]; o[4] = v[3]; o[5] = v[4];
    o[6] = v[2]; o[7] = v[4]; o[8] = v[5];
}

void launch_expand_V(const DeviceProblem &d, const double *V6, double *V9, cudaStream_t s)
{
    if (d.np == 0) return;
    if (d.prec == PSBA_PREC_FP64)
        k_expand_V<double><<<ceil_div(d.np, 128), 128, 0, s>>>(d.np, V6, V9);
    else
        k_expand_V<float><<<ceil_div(d.np, 128), 128, 0, s>>>(d.np, (const float *)V6, V9);
    note_launch(1);
}

}  // namespace psba

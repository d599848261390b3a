/*
 * FP64 CPU oracle — restatement of the reference's LM / trust-region bundle
 * adjustment path.  TEST INFRASTRUCTURE ONLY (see psba_oracle.h).
 *
 * Every stage keeps the reference's arithmetic: the same expressions, the
 * same accumulation order (ascending point index for per-camera sums,
 * ascending camera index for per-point sums, ascending common point for the
 * Schur blocks, ascending parameter index for host reductions).  The
 * reference iterates dense (point x camera) grids and skips unobserved
 * pairs; here the same sums run over sparse index lists in the same order,
 * which gives the same floating-point result.
 *
 * Build: oracle/build.py (gcc -O2 -ffp-contract=off -fopenmp).  OpenMP only
 * distributes independent outputs; no reduction changes order with the
 * thread count.
 */
#include "psba_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define CNP 6
#define PNP 3
#define MNP 2

void orc_default_opts(orc_opts *o)
{
    o->tau = 1e-3;          /* PSBA_INIT_MU     psba.h:6 */
    o->stop_thresh = 1e-12; /* PSBA_STOP_THRESH psba.h:7 */
    o->eps = 1e-12;         /* PSBA_EPSILON     psba.h:8 */
    o->eps2 = 1e-12;        /* PSBA_EPSILON2    psba.h:9 */
    o->max_iter = 50;       /* levmar.cpp:100, trust_region.cpp:112 */
    o->allow_switch = 1;
    o->solve_mode = 0;
    o->n_threads = 1;
}

/* ------------------------------------------------------------------------ */
/* index lists (replace generate_idxs' dense blk_idx / comm3DIdx, misc.cpp:178-218) */

typedef struct {
    int nc, np, no;
    int *pt_start;         /* np+1, observations of point i: [pt_start[i], pt_start[i+1]) */
    int *cam_start;        /* nc+1 */
    int *cam_obs;          /* observations sorted by (camera, point) */
    long long *pair_start; /* (k,l), k>=l, slot k*(k+1)/2+l; entries in ascending point */
    int *pair_a;           /* observation of camera k */
    int *pair_b;           /* observation of camera l */
} orc_index;

static void idx_free(orc_index *ix)
{
    free(ix->pt_start);
    free(ix->cam_start);
    free(ix->cam_obs);
    free(ix->pair_start);
    free(ix->pair_a);
    free(ix->pair_b);
    memset(ix, 0, sizeof(*ix));
}

static int idx_build(const orc_problem *p, orc_index *ix, int with_pairs)
{
    memset(ix, 0, sizeof(*ix));
    ix->nc = p->nc;
    ix->np = p->np;
    ix->no = p->no;
    ix->pt_start = (int *)calloc((size_t)p->np + 1, sizeof(int));
    ix->cam_start = (int *)calloc((size_t)p->nc + 1, sizeof(int));
    ix->cam_obs = (int *)malloc(sizeof(int) * (size_t)(p->no > 0 ? p->no : 1));
    if (!ix->pt_start || !ix->cam_start || !ix->cam_obs) return -1;
    for (int o = 0; o < p->no; ++o) {
        ix->pt_start[p->obs_pt[o] + 1]++;
        ix->cam_start[p->obs_cam[o] + 1]++;
    }
    for (int i = 0; i < p->np; ++i) ix->pt_start[i + 1] += ix->pt_start[i];
    for (int j = 0; j < p->nc; ++j) ix->cam_start[j + 1] += ix->cam_start[j];
    {
        int *fill = (int *)malloc(sizeof(int) * ((size_t)p->nc + 1));
        memcpy(fill, ix->cam_start, sizeof(int) * ((size_t)p->nc + 1));
        for (int o = 0; o < p->no; ++o) ix->cam_obs[fill[p->obs_cam[o]]++] = o;
        free(fill);
    }
    if (!with_pairs) return 0;
    {
        size_t npair = (size_t)p->nc * (p->nc + 1) / 2;
        long long *cnt = (long long *)calloc(npair + 1, sizeof(long long));
        for (int i = 0; i < p->np; ++i)
            for (int a = ix->pt_start[i]; a < ix->pt_start[i + 1]; ++a)
                for (int b = ix->pt_start[i]; b < ix->pt_start[i + 1]; ++b) {
                    int k = p->obs_cam[a], l = p->obs_cam[b];
                    if (l <= k) cnt[(size_t)k * (k + 1) / 2 + l + 1]++;
                }
        for (size_t s = 0; s < npair; ++s) cnt[s + 1] += cnt[s];
        ix->pair_start = cnt;
        ix->pair_a = (int *)malloc(sizeof(int) * (size_t)(cnt[npair] > 0 ? cnt[npair] : 1));
        ix->pair_b = (int *)malloc(sizeof(int) * (size_t)(cnt[npair] > 0 ? cnt[npair] : 1));
        long long *fill = (long long *)malloc(sizeof(long long) * (npair + 1));
        memcpy(fill, cnt, sizeof(long long) * (npair + 1));
        for (int i = 0; i < p->np; ++i)
            for (int a = ix->pt_start[i]; a < ix->pt_start[i + 1]; ++a)
                for (int b = ix->pt_start[i]; b < ix->pt_start[i + 1]; ++b) {
                    int k = p->obs_cam[a], l = p->obs_cam[b];
                    if (l <= k) {
                        long long at = fill[(size_t)k * (k + 1) / 2 + l]++;
                        ix->pair_a[at] = a;
                        ix->pair_b[at] = b;
                    }
                }
        free(fill);
    }
    return 0;
}

long long orc_pair_count(const orc_problem *p)
{
    orc_index ix;
    idx_build(p, &ix, 1);
    long long n = ix.pair_start[(size_t)p->nc * (p->nc + 1) / 2];
    idx_free(&ix);
    return n;
}

/* ------------------------------------------------------------------------ */
/* a1/a2: projection.  compute_exQT.cl:33-69, levmar_func_cpu.cpp:185-223.
 * The camera rotation is the Hamilton product q(v) (x) q0 with
 * q(v) = (sqrt(1-|v|^2), v); the point is rotated by the sandwich
 * q (0,X) q*, translated, and projected with K = [fx cx cy ar skew]:
 *   x = (fx Xc + skew Yc + cx Zc) / Zc,   y = (fx ar Yc + cy Zc) / Zc.      */

/* The additions are grouped as in compute_exQT.cl:82-107 so that this stage
 * reproduces the reference bit for bit. */
static void compose_quat(const double *q0, const double *v, double q[4])
{
    double sl = sqrt(1 - v[0] * v[0] - v[1] * v[1] - v[2] * v[2]);
    double s0 = q0[0], a1 = q0[1], a2 = q0[2], a3 = q0[3];
    q[0] = sl * s0 - (a1 * v[0] + a2 * v[1] + a3 * v[2]);
    q[1] = s0 * v[0] + sl * a1 + a3 * v[1] - a2 * v[2];
    q[2] = s0 * v[1] + sl * a2 + a1 * v[2] - a3 * v[0];
    q[3] = s0 * v[2] + sl * a3 + a2 * v[0] - a1 * v[1];
}

/* Xc = q (0,X) conj(q) + t, for a (not necessarily unit) quaternion q:
 * m = q (0,X), then the vector part of m conj(q). */
static void quat_rotate_t(const double q[4], const double X[3], const double *t, double out[3])
{
    double s = q[0], a = q[1], b = q[2], c = q[3];
    double m0 = -X[0] * a - b * X[1] - c * X[2];
    double m1 = s * X[0] + b * X[2] - c * X[1];
    double m2 = X[1] * s + c * X[0] - X[2] * a;
    double m3 = s * X[2] + X[1] * a - b * X[0];
    out[0] = -a * m0 + s * m1 - m2 * c + b * m3 + t[0];
    out[1] = -b * m0 + s * m2 - m3 * a + c * m1 + t[1];
    out[2] = -m0 * c + s * m3 - b * m1 + a * m2 + t[2];
}

static int cnp_of(const orc_problem *p) { return p->cnp > 0 ? p->cnp : CNP; }

/* Variable intrinsics (cnp 11 / 16; no reference counterpart).  Camera j's
 * parameters: v (3), t (3), K = fx, cx, cy, ar, skew (5), and for cnp 16
 * distortion kc = k1, k2, p1, p2, k3 (5).  With x = Xc/Zc, y = Yc/Zc,
 * r2 = x^2 + y^2:
 *   radial = 1 + k1 r2 + k2 r2^2 + k3 r2^3,
 *   xd = radial x + 2 p1 x y + p2 (r2 + 2 x^2),
 *   yd = radial y + p1 (r2 + 2 y^2) + 2 p2 x y,
 *   u = fx xd + skew yd + cx,   v = fx ar yd + cy.
 * Without distortion (cnp 11) the projection is evaluated exactly as for
 * fixed K: u = (fx Xc + skew Yc + cx Zc) / Zc, v = (fx ar Yc + cy Zc) / Zc. */
static void distort(const double *kc, double x, double y, double *xd, double *yd)
{
    double r2 = x * x + y * y;
    double radial = 1.0 + r2 * (kc[0] + r2 * (kc[1] + r2 * kc[4]));
    *xd = radial * x + 2.0 * kc[2] * x * y + kc[3] * (r2 + 2.0 * x * x);
    *yd = radial * y + kc[2] * (r2 + 2.0 * y * y) + 2.0 * kc[3] * x * y;
}

static void project_v(const double *q0, const double *cam, int cnp, const double *X, double *xy)
{
    double q[4], Xc[3];
    compose_quat(q0, cam, q);
    quat_rotate_t(q, X, cam + 3, Xc);
    const double *K = cam + 6;
    double iz = 1 / Xc[2];
    if (cnp == 11) {
        xy[0] = (K[0] * Xc[0] + K[4] * Xc[1] + K[1] * Xc[2]) * iz;
        xy[1] = (K[0] * K[3] * Xc[1] + K[2] * Xc[2]) * iz;
        return;
    }
    double xd, yd;
    distort(cam + 11, Xc[0] * iz, Xc[1] * iz, &xd, &yd);
    xy[0] = K[0] * xd + K[4] * yd + K[1];
    xy[1] = K[0] * K[3] * yd + K[2];
}

static void project(const double *K, const double q[4], const double *t, const double *X,
                    double *xy, double Xc[3])
{
    quat_rotate_t(q, X, t, Xc);
    double iz = 1 / Xc[2];
    xy[0] = (K[0] * Xc[0] + K[4] * Xc[1] + K[1] * Xc[2]) * iz;
    xy[1] = (K[0] * K[3] * Xc[1] + K[2] * Xc[2]) * iz;
}

void orc_residual(const orc_problem *p, const double *cams, const double *pts, double *ex)
{
    const int cnp = cnp_of(p);
#pragma omp parallel for schedule(static)
    for (int o = 0; o < p->no; ++o) {
        int i = p->obs_pt[o], j = p->obs_cam[o];
        double q[4], xy[2], Xc[3];
        if (cnp > 6) {
            project_v(p->q0 + 4 * j, cams + (size_t)cnp * j, cnp, pts + PNP * i, xy);
        } else {
            compose_quat(p->q0 + 4 * j, cams + CNP * j, q);
            project(p->K + 5 * j, q, cams + CNP * j + 3, pts + PNP * i, xy, Xc);
        }
        double e0 = p->meas[2 * o] - xy[0], e1 = p->meas[2 * o + 1] - xy[1];
        if (p->wt) {
            const double *w = p->wt + 3 * (size_t)o;
            double t0 = w[0] * e0 + w[1] * e1;
            e1 = w[2] * e1;
            e0 = t0;
        }
        ex[2 * o] = e0;
        ex[2 * o + 1] = e1;
    }
}

/* compute_L2_sq, misc.cpp:151-157 (sequential order) */
double orc_sumsq(int n, const double *x)
{
    double s = 0;
    for (int i = 0; i < n; ++i) s += x[i] * x[i];
    return s;
}

static double dotp(int n, const double *a, const double *b) /* dotProduct, misc.cpp:162-169 */
{
    double s = 0.0;
    for (int i = 0; i < n; ++i) s += a[i] * b[i];
    return s;
}

/* ------------------------------------------------------------------------ */
/* a3/a4: analytic Jacobian of the projection, the quantity that
 * compute_jacobiQT.cl:23-140 and levmar_func_cpu.cpp:227-455 evaluate in
 * expanded form.  Here it is the chain rule:
 *   d(x,y)/dXc  (2x3)  from the pinhole + skew + aspect model,
 *   dXc/dq      (3x4)  of the sandwich f(q) = (s^2-|v|^2)X + 2(v.X)v + 2s(v x X),
 *   dq/dv_l     (4x3)  of q = q(v_l) (x) q0 with s_l = sqrt(1-|v_l|^2),
 *   dXc/dt = I, dXc/dX = (s^2-|v|^2)I + 2vv^T + 2s[v]x.
 * A = [d(x,y)/dXc * dXc/dv_l | d(x,y)/dXc],  B = d(x,y)/dXc * dXc/dX.        */
static void jac_one(const double *K, const double *q0, const double *cam, const double *X,
                    double *A /*2x6*/, double *B /*2x3*/)
{
    const double *vl = cam;
    double q[4], xy[2], Xc[3];
    compose_quat(q0, vl, q);
    project(K, q, cam + 3, X, xy, Xc);
    double s = q[0], v[3] = {q[1], q[2], q[3]};
    double iz = 1.0 / Xc[2];
    double fx = K[0], sk = K[4], fy = K[0] * K[3];
    double P[2][3];
    P[0][0] = fx * iz;
    P[0][1] = sk * iz;
    P[0][2] = -(fx * Xc[0] + sk * Xc[1]) * iz * iz;
    P[1][0] = 0.0;
    P[1][1] = fy * iz;
    P[1][2] = -fy * Xc[1] * iz * iz;

    double vX = v[0] * X[0] + v[1] * X[1] + v[2] * X[2];
    double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double vxX[3] = {v[1] * X[2] - v[2] * X[1], v[2] * X[0] - v[0] * X[2], v[0] * X[1] - v[1] * X[0]};
    /* df/dq: column 0 w.r.t. s, columns 1..3 w.r.t. v_m */
    double F[3][4];
    for (int r = 0; r < 3; ++r) F[r][0] = 2.0 * s * X[r] + 2.0 * vxX[r];
    for (int m = 0; m < 3; ++m) {
        double em_x_X[3] = {0, 0, 0}; /* e_m x X */
        if (m == 0) { em_x_X[1] = -X[2]; em_x_X[2] = X[1]; }
        if (m == 1) { em_x_X[0] = X[2]; em_x_X[2] = -X[0]; }
        if (m == 2) { em_x_X[0] = -X[1]; em_x_X[1] = X[0]; }
        for (int r = 0; r < 3; ++r)
            F[r][m + 1] = -2.0 * v[m] * X[r] + 2.0 * X[m] * v[r] + (r == m ? 2.0 * vX : 0.0) +
                          2.0 * s * em_x_X[r];
    }
    /* dq/dv_l */
    double sl = sqrt(1.0 - vl[0] * vl[0] - vl[1] * vl[1] - vl[2] * vl[2]);
    double s0 = q0[0], a[3] = {q0[1], q0[2], q0[3]};
    double D[4][3];
    for (int m = 0; m < 3; ++m) {
        double ds = -vl[m] / sl;
        double em_x_a[3] = {0, 0, 0}; /* e_m x a */
        if (m == 0) { em_x_a[1] = -a[2]; em_x_a[2] = a[1]; }
        if (m == 1) { em_x_a[0] = a[2]; em_x_a[2] = -a[0]; }
        if (m == 2) { em_x_a[0] = -a[1]; em_x_a[1] = a[0]; }
        D[0][m] = s0 * ds - a[m];
        for (int r = 0; r < 3; ++r) D[r + 1][m] = a[r] * ds + (r == m ? s0 : 0.0) + em_x_a[r];
    }
    double G[3][3]; /* dXc/dv_l */
    for (int r = 0; r < 3; ++r)
        for (int m = 0; m < 3; ++m)
            G[r][m] = F[r][0] * D[0][m] + F[r][1] * D[1][m] + F[r][2] * D[2][m] + F[r][3] * D[3][m];
    double R[3][3];
    double d = s * s - vv;
    R[0][0] = d + 2 * v[0] * v[0];
    R[0][1] = 2 * v[0] * v[1] - 2 * s * v[2];
    R[0][2] = 2 * v[0] * v[2] + 2 * s * v[1];
    R[1][0] = 2 * v[1] * v[0] + 2 * s * v[2];
    R[1][1] = d + 2 * v[1] * v[1];
    R[1][2] = 2 * v[1] * v[2] - 2 * s * v[0];
    R[2][0] = 2 * v[2] * v[0] - 2 * s * v[1];
    R[2][1] = 2 * v[2] * v[1] + 2 * s * v[0];
    R[2][2] = d + 2 * v[2] * v[2];
    for (int r = 0; r < 2; ++r) {
        for (int m = 0; m < 3; ++m) {
            A[r * 6 + m] = P[r][0] * G[0][m] + P[r][1] * G[1][m] + P[r][2] * G[2][m];
            A[r * 6 + 3 + m] = P[r][m];
            B[r * 3 + m] = P[r][0] * R[0][m] + P[r][1] * R[1][m] + P[r][2] * R[2][m];
        }
    }
}

/* Jacobian of the variable-intrinsics model, 2 x cnp (camera) and 2 x 3
 * (point).  With P = d(u,v)/d(xd,yd) = [[fx, skew], [0, fx ar]],
 * Dd = d(xd,yd)/d(x,y) (identity without distortion) and
 * N = d(x,y)/dXc = [[1/Zc, 0, -x/Zc], [0, 1/Zc, -y/Zc]], the chain
 * H = P Dd N replaces d(x,y)/dXc of jac_one; the pose and point columns are
 * then H dXc/dv_l, H, H dXc/dX as there.  Intrinsics columns:
 * du/dfx = xd, dv/dfx = ar yd; du/dcx = 1; dv/dcy = 1; dv/dar = fx yd;
 * du/dskew = yd.  Distortion columns: P d(xd,yd)/dkc.                       */
static void jac_one_v(const double *q0, const double *cam, int cnp, const double *X, double *A, double *B)
{
    const double *vl = cam, *K = cam + 6;
    double q[4], Xc[3];
    compose_quat(q0, vl, q);
    quat_rotate_t(q, X, cam + 3, Xc);
    double iz = 1.0 / Xc[2], x = Xc[0] * iz, y = Xc[1] * iz;
    double fx = K[0], sk = K[4], ar = K[3], fy = K[0] * K[3];
    double Dd[2][2] = {{1.0, 0.0}, {0.0, 1.0}}, xd = x, yd = y, r2 = x * x + y * y;
    const double *kc = cam + 11;
    if (cnp == 16) {
        distort(kc, x, y, &xd, &yd);
        double radial = 1.0 + r2 * (kc[0] + r2 * (kc[1] + r2 * kc[4]));
        double dr = kc[0] + r2 * (2.0 * kc[1] + 3.0 * kc[4] * r2); /* d radial / d r2 */
        Dd[0][0] = radial + 2.0 * x * x * dr + 2.0 * kc[2] * y + 6.0 * kc[3] * x;
        Dd[0][1] = 2.0 * x * y * dr + 2.0 * kc[2] * x + 2.0 * kc[3] * y;
        Dd[1][0] = 2.0 * x * y * dr + 2.0 * kc[2] * x + 2.0 * kc[3] * y;
        Dd[1][1] = radial + 2.0 * y * y * dr + 6.0 * kc[2] * y + 2.0 * kc[3] * x;
    }
    double PD[2][2] = {{fx * Dd[0][0] + sk * Dd[1][0], fx * Dd[0][1] + sk * Dd[1][1]},
                       {fy * Dd[1][0], fy * Dd[1][1]}};
    double H[2][3];
    for (int r = 0; r < 2; ++r) {
        H[r][0] = PD[r][0] * iz;
        H[r][1] = PD[r][1] * iz;
        H[r][2] = -(PD[r][0] * x + PD[r][1] * y) * iz;
    }
    /* dXc/dv_l and dXc/dX as in jac_one */
    double s = q[0], v[3] = {q[1], q[2], q[3]};
    double vX = v[0] * X[0] + v[1] * X[1] + v[2] * X[2];
    double vv = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    double vxX[3] = {v[1] * X[2] - v[2] * X[1], v[2] * X[0] - v[0] * X[2], v[0] * X[1] - v[1] * X[0]};
    double F[3][4];
    for (int r = 0; r < 3; ++r) F[r][0] = 2.0 * s * X[r] + 2.0 * vxX[r];
    for (int m = 0; m < 3; ++m) {
        double em_x_X[3] = {0, 0, 0};
        if (m == 0) { em_x_X[1] = -X[2]; em_x_X[2] = X[1]; }
        if (m == 1) { em_x_X[0] = X[2]; em_x_X[2] = -X[0]; }
        if (m == 2) { em_x_X[0] = -X[1]; em_x_X[1] = X[0]; }
        for (int r = 0; r < 3; ++r)
            F[r][m + 1] = -2.0 * v[m] * X[r] + 2.0 * X[m] * v[r] + (r == m ? 2.0 * vX : 0.0) +
                          2.0 * s * em_x_X[r];
    }
    double sl = sqrt(1.0 - vl[0] * vl[0] - vl[1] * vl[1] - vl[2] * vl[2]);
    double s0 = q0[0], a[3] = {q0[1], q0[2], q0[3]};
    double D[4][3];
    for (int m = 0; m < 3; ++m) {
        double ds = -vl[m] / sl;
        double em_x_a[3] = {0, 0, 0};
        if (m == 0) { em_x_a[1] = -a[2]; em_x_a[2] = a[1]; }
        if (m == 1) { em_x_a[0] = a[2]; em_x_a[2] = -a[0]; }
        if (m == 2) { em_x_a[0] = -a[1]; em_x_a[1] = a[0]; }
        D[0][m] = s0 * ds - a[m];
        for (int r = 0; r < 3; ++r) D[r + 1][m] = a[r] * ds + (r == m ? s0 : 0.0) + em_x_a[r];
    }
    double G[3][3];
    for (int r = 0; r < 3; ++r)
        for (int m = 0; m < 3; ++m)
            G[r][m] = F[r][0] * D[0][m] + F[r][1] * D[1][m] + F[r][2] * D[2][m] + F[r][3] * D[3][m];
    double R[3][3];
    double d = s * s - vv;
    R[0][0] = d + 2 * v[0] * v[0];
    R[0][1] = 2 * v[0] * v[1] - 2 * s * v[2];
    R[0][2] = 2 * v[0] * v[2] + 2 * s * v[1];
    R[1][0] = 2 * v[1] * v[0] + 2 * s * v[2];
    R[1][1] = d + 2 * v[1] * v[1];
    R[1][2] = 2 * v[1] * v[2] - 2 * s * v[0];
    R[2][0] = 2 * v[2] * v[0] - 2 * s * v[1];
    R[2][1] = 2 * v[2] * v[1] + 2 * s * v[0];
    R[2][2] = d + 2 * v[2] * v[2];
    for (int r = 0; r < 2; ++r)
        for (int m = 0; m < 3; ++m) {
            A[r * cnp + m] = H[r][0] * G[0][m] + H[r][1] * G[1][m] + H[r][2] * G[2][m];
            A[r * cnp + 3 + m] = H[r][m];
            B[r * 3 + m] = H[r][0] * R[0][m] + H[r][1] * R[1][m] + H[r][2] * R[2][m];
        }
    /* intrinsics fx, cx, cy, ar, skew */
    A[6] = xd;       A[cnp + 6] = ar * yd;
    A[7] = 1.0;      A[cnp + 7] = 0.0;
    A[8] = 0.0;      A[cnp + 8] = 1.0;
    A[9] = 0.0;      A[cnp + 9] = fx * yd;
    A[10] = yd;      A[cnp + 10] = 0.0;
    if (cnp == 16) {
        double r4 = r2 * r2, r6 = r4 * r2;
        double dxd[5] = {x * r2, x * r4, 2.0 * x * y, r2 + 2.0 * x * x, x * r6};
        double dyd[5] = {y * r2, y * r4, r2 + 2.0 * y * y, 2.0 * x * y, y * r6};
        for (int k = 0; k < 5; ++k) {
            A[11 + k] = fx * dxd[k] + sk * dyd[k];
            A[cnp + 11 + k] = fy * dyd[k];
        }
    }
}

void orc_jacobian(const orc_problem *p, const double *cams, const double *pts, double *JA, double *JB)
{
    const int cnp = cnp_of(p);
#pragma omp parallel for schedule(static)
    for (int o = 0; o < p->no; ++o) {
        int i = p->obs_pt[o], j = p->obs_cam[o];
        double *A = JA + 2 * (size_t)cnp * o, *B = JB + 6 * (size_t)o;
        if (cnp > 6)
            jac_one_v(p->q0 + 4 * j, cams + (size_t)cnp * j, cnp, pts + PNP * i, A, B);
        else
            jac_one(p->K + 5 * j, p->q0 + 4 * j, cams + CNP * j, pts + PNP * i, A, B);
        if (p->wt) {  /* rows <- L rows */
            const double *w = p->wt + 3 * (size_t)o;
            for (int m = 0; m < cnp; ++m) {
                double a0 = A[m], a1 = A[cnp + m];
                A[m] = w[0] * a0 + w[1] * a1;
                A[cnp + m] = w[2] * a1;
            }
            for (int m = 0; m < PNP; ++m) {
                double b0 = B[m], b1 = B[PNP + m];
                B[m] = w[0] * b0 + w[1] * b1;
                B[PNP + m] = w[2] * b1;
            }
        }
    }
}

/* ------------------------------------------------------------------------ */
/* a5-a8: U, V, W, g.  compute_U.cl:21-34, compute_V.cl:24-37,
 * compute_Wblks.cl:25-33, compute_g.cl:25-59.  coeff multiplies the sum.   */
static void normal_blocks_ix(const orc_problem *p, const orc_index *ix, const double *JA,
                             const double *JB, const double *ex, double coeff, double *U, double *V,
                             double *W, double *g, double *UVdiag)
{
    int nc = p->nc, np = p->np;
    const int cnp = cnp_of(p);
#pragma omp parallel for schedule(dynamic, 1)
    for (int j = 0; j < nc; ++j) {
        for (int r = 0; r < cnp; ++r)
            for (int c = 0; c < cnp; ++c) {
                double sum = 0;
                for (int e = ix->cam_start[j]; e < ix->cam_start[j + 1]; ++e) {
                    const double *A = JA + 2 * (size_t)cnp * ix->cam_obs[e];
                    sum = sum + A[r] * A[c] + A[cnp + r] * A[cnp + c];
                }
                sum = coeff * sum;
                U[(size_t)j * cnp * cnp + r * cnp + c] = sum;
                if (r == c) UVdiag[j * cnp + r] = sum;
            }
        for (int k = 0; k < cnp; ++k) {
            double sum = 0;
            for (int e = ix->cam_start[j]; e < ix->cam_start[j + 1]; ++e) {
                int o = ix->cam_obs[e];
                const double *A = JA + 2 * (size_t)cnp * o;
                sum = sum + A[k] * ex[2 * (size_t)o] + A[k + cnp] * ex[2 * (size_t)o + 1];
            }
            g[j * cnp + k] = coeff * sum;
        }
    }
#pragma omp parallel for schedule(static)
    for (int i = 0; i < np; ++i) {
        for (int r = 0; r < PNP; ++r)
            for (int c = 0; c < PNP; ++c) {
                double sum = 0;
                for (int o = ix->pt_start[i]; o < ix->pt_start[i + 1]; ++o) {
                    const double *B = JB + 6 * (size_t)o;
                    sum = sum + B[r] * B[c] + B[PNP + r] * B[PNP + c];
                }
                sum = coeff * sum;
                V[(size_t)i * 9 + r * 3 + c] = sum;
                if (r == c) UVdiag[(size_t)nc * cnp + i * PNP + r] = sum;
            }
        for (int k = 0; k < PNP; ++k) {
            double sum = 0;
            for (int o = ix->pt_start[i]; o < ix->pt_start[i + 1]; ++o) {
                const double *B = JB + 6 * (size_t)o;
                sum = sum + B[k] * ex[2 * (size_t)o] + B[k + PNP] * ex[2 * (size_t)o + 1];
            }
            g[(size_t)nc * cnp + i * PNP + k] = coeff * sum;
        }
    }
#pragma omp parallel for schedule(static)
    for (int o = 0; o < p->no; ++o) {
        const double *A = JA + 2 * (size_t)cnp * o, *B = JB + 6 * (size_t)o;
        for (int r = 0; r < cnp; ++r)
            for (int c = 0; c < PNP; ++c) {
                double sum = A[r] * B[c] + A[cnp + r] * B[PNP + c];
                W[(size_t)o * 3 * cnp + r * 3 + c] = coeff * sum;
            }
    }
}

void orc_normal_blocks(const orc_problem *p, const double *JA, const double *JB, const double *ex,
                       double coeff, double *U, double *V, double *W, double *g, double *UVdiag)
{
    orc_index ix;
    idx_build(p, &ix, 0);
    normal_blocks_ix(p, &ix, JA, JB, ex, coeff, U, V, W, g, UVdiag);
    idx_free(&ix);
}

/* ------------------------------------------------------------------------ */
/* a11: 3x3 inverse of V_i + mu I by cofactors, compute_Vinv.cl:29-86.
 * Reads the upper triangle and the (damped) diagonal; writes the symmetric
 * inverse.  The branch for |T| < 1e-16 restates the reference's pivoted
 * elimination (compute_Vinv.cl:31-73) on the symmetric matrix; its
 * `a[0, 0] != 0` test (:41) is a comma expression that is always true, so
 * the elimination step always runs.                                          */
static void vinv_one(const double *Vi, double mu, double *out)
{
    double a11 = Vi[0] + mu, a12 = Vi[1], a13 = Vi[2];
    double a22 = Vi[4] + mu, a23 = Vi[5];
    double a33 = Vi[8] + mu;
    double a21 = a12, a31 = a13, a32 = a23;
    double T = (a33 * a12 * a12 - 2 * a12 * a13 * a23 + a22 * a13 * a13 + a11 * a23 * a23 -
                a11 * a22 * a33);
    double i00, i10, i11, i20, i21, i22;
    if (fabs(T) < 1e-16) {
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
        i00 = (a22 * a33 - a23 * a32) / T;
        i10 = -(a21 * a33 - a23 * a31) / T;
        i11 = (a11 * a33 - a13 * a31) / T;
        i20 = (a21 * a32 - a22 * a31) / T;
        i21 = -(a11 * a32 - a12 * a31) / T;
        i22 = (a11 * a22 - a12 * a21) / T;
    } else {
        i00 = -(-a23 * a23 + a22 * a33) / T;
        i10 = -(a13 * a23 - a12 * a33) / T;
        i11 = -(-a13 * a13 + a11 * a33) / T;
        i20 = -(a12 * a23 - a13 * a22) / T;
        i21 = -(a12 * a13 - a11 * a23) / T;
        i22 = -(-a12 * a12 + a11 * a22) / T;
    }
    out[0] = i00; out[1] = i10; out[2] = i20;
    out[3] = i10; out[4] = i11; out[5] = i21;
    out[6] = i20; out[7] = i21; out[8] = i22;
}

void orc_vinv(int np, const double *V, double mu, double *Vinv)
{
#pragma omp parallel for schedule(static)
    for (int i = 0; i < np; ++i) vinv_one(V + 9 * (size_t)i, mu, Vinv + 9 * (size_t)i);
}

/* a12: Y_ij = W_ij V_i^-1, compute_Yblks.cl:26-37 */
void orc_yblocks(const orc_problem *p, const double *W, const double *Vinv, double *Y)
{
    const int cnp = cnp_of(p);
#pragma omp parallel for schedule(static)
    for (int o = 0; o < p->no; ++o) {
        const double *Wo = W + 3 * (size_t)cnp * o, *Vi = Vinv + 9 * (size_t)p->obs_pt[o];
        double *Yo = Y + 3 * (size_t)cnp * o;
        for (int r = 0; r < cnp; ++r)
            for (int c = 0; c < PNP; ++c)
                Yo[r * 3 + c] = Wo[r * 3] * Vi[0 * 3 + c] + Wo[r * 3 + 1] * Vi[1 * 3 + c] +
                                Wo[r * 3 + 2] * Vi[2 * 3 + c];
    }
}

/* a13: S_kl = delta_kl (U_k + mu I) - sum_i Y_ik W_il^T, compute_S.cl:39-77,
 * common points in ascending order (misc.cpp:189-211).  Lower triangle only
 * (the Cholesky of SPD_inv.cl reads nothing else).                           */
static void schur_ix(const orc_problem *p, const orc_index *ix, const double *U, double mu,
                     const double *Y, const double *W, double *S)
{
    int nc = p->nc;
    const int cnp = cnp_of(p);
    size_t N = (size_t)nc * cnp;
    long long npair = (long long)nc * (nc + 1) / 2;
#pragma omp parallel for schedule(dynamic, 4)
    for (long long s = 0; s < npair; ++s) {
        int k = (int)((sqrt(8.0 * (double)s + 1.0) - 1.0) / 2.0);
        while ((long long)k * (k + 1) / 2 > s) --k;
        while ((long long)(k + 1) * (k + 2) / 2 <= s) ++k;
        int l = (int)(s - (long long)k * (k + 1) / 2);
        long long b = ix->pair_start[s], e = ix->pair_start[s + 1];
        for (int r = 0; r < cnp; ++r)
            for (int c = 0; c < cnp; ++c) {
                if (k == l && c > r) continue;
                double sum = 0;
                for (long long t = b; t < e; ++t) {
                    const double *y = Y + 3 * (size_t)cnp * ix->pair_a[t] + r * 3;
                    const double *w = W + 3 * (size_t)cnp * ix->pair_b[t] + c * 3;
                    sum += (y[0] * w[0] + y[1] * w[1] + y[2] * w[2]);
                }
                double val;
                if (k == l)
                    val = (r == c ? U[(size_t)k * cnp * cnp + r * cnp + c] + mu : U[(size_t)k * cnp * cnp + r * cnp + c]) - sum;
                else
                    val = -sum;
                S[((size_t)k * cnp + r) * N + (size_t)l * cnp + c] = val;
            }
    }
}

void orc_schur(const orc_problem *p, const double *U, double mu, const double *Y, const double *W,
               double *S)
{
    orc_index ix;
    idx_build(p, &ix, 1);
    schur_ix(p, &ix, U, mu, Y, W, S);
    idx_free(&ix);
}

/* a14: ea = ga - sum_i Y_ij gb_i, compute_ea.cl:21-36 */
static void ea_ix(const orc_problem *p, const orc_index *ix, const double *Y, const double *g,
                  double *ea)
{
    int nc = p->nc;
    const int cnp = cnp_of(p);
    const double *gb = g + (size_t)nc * cnp;
    for (int j = 0; j < nc; ++j)
        for (int r = 0; r < cnp; ++r) {
            double sum = 0;
            for (int e = ix->cam_start[j]; e < ix->cam_start[j + 1]; ++e) {
                int o = ix->cam_obs[e];
                const double *y = Y + 3 * (size_t)cnp * o + r * 3;
                const double *b = gb + 3 * (size_t)p->obs_pt[o];
                sum = sum + y[0] * b[0] + y[1] * b[1] + y[2] * b[2];
            }
            ea[j * cnp + r] = g[j * cnp + r] - sum;
        }
}

void orc_ea(const orc_problem *p, const double *Y, const double *g, double *ea)
{
    orc_index ix;
    idx_build(p, &ix, 0);
    ea_ix(p, &ix, Y, g, ea);
    idx_free(&ix);
}

/* ------------------------------------------------------------------------ */
/* a15/a16: SPD inverse and S^-1 ea, SPD_inv.cl + cl_spdinv.cpp:18-40.
 * 3x3-block right-looking Cholesky (SPD_inv.cl:20-239): for block column j,
 * T_ij = A_ij - sum_{k<j} L_ik L_jk^T for i >= j; the diagonal block is
 * factored in closed form (:60-111) together with its inverse (:115-159);
 * L_ij = T_ij L_jj^-T below it.  Any non-finite value in the diagonal
 * block, its inverse or the pivots stops the chain with status 1.
 * Then X = L^-1 diagonal by diagonal (kern_trigMat_inv, :248-328) and
 * S^-1 = X^T X (kern_trigMat_mul, :343-385).                                */

static int blk_chol_diag(const double *T /*3x3*/, double *L /*6*/, double *Li /*3x3*/)
{
    int bad = 0;
    L[0] = sqrt(T[0]);
    L[1] = T[3] / sqrt(T[0]);
    L[2] = sqrt(T[4] - T[3] * T[3] / T[0]);
    L[3] = T[6] / sqrt(T[0]);
    L[4] = sqrt(T[0] / (T[0] * T[4] - T[3] * T[3])) * (T[7] - T[3] * T[6] / T[0]);
    {
        double t1 = -T[8] * T[3] * T[3];
        double t2 = 2 * T[7] * T[3] * T[6];
        double t3 = -T[4] * T[6] * T[6];
        double t4 = T[0] * (T[4] * T[8] - T[7] * T[7]);
        double t5 = -T[3] * T[3] + T[0] * T[4];
        L[5] = sqrt((t1 + t2 + t3 + t4) / t5);
    }
    for (int k = 0; k < 6; ++k)
        if (!isfinite(L[k])) bad = 1;
    Li[0] = 1 / L[0];
    Li[1] = 0;
    Li[2] = 0;
    Li[3] = -L[1] / (L[0] * L[2]);
    Li[4] = 1 / L[2];
    Li[5] = 0;
    Li[6] = (L[1] * L[4] - L[2] * L[3]) / (L[0] * L[2] * L[5]);
    Li[7] = -L[4] / (L[2] * L[5]);
    Li[8] = 1 / L[5];
    for (int k = 0; k < 9; ++k)
        if (!isfinite(Li[k])) bad = 1;
    return bad;
}

/* Block Cholesky in place on the lower triangle of S (n % 3 == 0).  On
 * return the lower triangle holds L (upper zeroed) and dinv holds the
 * 3x3 L_jj^-1 blocks.  Returns 0 on success, 1 on failure.                   */
static int blk_cholesky(int n, double *S, double *dinv)
{
    int nb = n / 3;
    for (int j = 0; j < nb; ++j) {
        /* T_ij for i >= j (kern_cholesky) */
#pragma omp parallel for schedule(static)
        for (int i = j; i < nb; ++i)
            for (int u = 0; u < 3; ++u)
                for (int v = 0; v < 3; ++v) {
                    size_t at = (size_t)(i * 3 + u) * n + j * 3 + v;
                    double sum = S[at];
                    const double *li = S + (size_t)(i * 3 + u) * n;
                    const double *lj = S + (size_t)(j * 3 + v) * n;
                    for (int k = 0; k < j; ++k)
                        sum -= (li[3 * k] * lj[3 * k] + li[3 * k + 1] * lj[3 * k + 1] +
                                li[3 * k + 2] * lj[3 * k + 2]);
                    S[at] = sum;
                }
        double T[9], L[6];
        for (int u = 0; u < 3; ++u)
            for (int v = 0; v < 3; ++v) T[u * 3 + v] = S[(size_t)(j * 3 + u) * n + j * 3 + v];
        int bad = blk_chol_diag(T, L, dinv + 9 * (size_t)j);
        double *d = S + (size_t)(j * 3) * n + j * 3;
        d[0] = L[0]; d[1] = 0; d[2] = 0;
        d[n] = L[1]; d[n + 1] = L[2]; d[n + 2] = 0;
        d[2 * n] = L[3]; d[2 * n + 1] = L[4]; d[2 * n + 2] = L[5];
        if (bad) return 1;
        /* L_ij = T_ij L_jj^-T for i > j (kern_cholesky_s2) */
        const double *Li = dinv + 9 * (size_t)j;
#pragma omp parallel for schedule(static)
        for (int i = j + 1; i < nb; ++i) {
            double Tij[9];
            for (int u = 0; u < 3; ++u)
                for (int w = 0; w < 3; ++w) Tij[u * 3 + w] = S[(size_t)(i * 3 + u) * n + j * 3 + w];
            for (int u = 0; u < 3; ++u)
                for (int v = 0; v < 3; ++v) {
                    double sum = 0.0;
                    sum += (Tij[u * 3] * Li[v * 3] + Tij[u * 3 + 1] * Li[v * 3 + 1] +
                            Tij[u * 3 + 2] * Li[v * 3 + 2]);
                    S[(size_t)(i * 3 + u) * n + j * 3 + v] = sum;
                    S[(size_t)(j * 3 + v) * n + i * 3 + u] = 0;
                }
        }
    }
    return 0;
}

/* Plain column Cholesky of the lower triangle (used where n % 3 != 0). */
static int col_cholesky(int n, double *S)
{
    for (int j = 0; j < n; ++j) {
        double d = S[(size_t)j * n + j];
        for (int k = 0; k < j; ++k) d -= S[(size_t)j * n + k] * S[(size_t)j * n + k];
        if (!(d > 0) || !isfinite(d)) return 1;
        double l = sqrt(d);
        S[(size_t)j * n + j] = l;
        for (int i = j + 1; i < n; ++i) {
            double s = S[(size_t)i * n + j];
            for (int k = 0; k < j; ++k) s -= S[(size_t)i * n + k] * S[(size_t)j * n + k];
            S[(size_t)i * n + j] = s / l;
            S[(size_t)j * n + i] = 0.0;
        }
    }
    return 0;
}

int orc_cholesky(int n, double *S)
{
    if (n % 3 != 0) return col_cholesky(n, S);
    double *dinv = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    int r = blk_cholesky(n, S, dinv);
    free(dinv);
    return r;
}

int orc_spd_inverse(int n, double *S)
{
    int nb = n / 3;
    double *dinv = (double *)malloc(sizeof(double) * 3 * (size_t)n);
    if (blk_cholesky(n, S, dinv)) {
        free(dinv);
        return 1;
    }
    /* X = L^-1 (lower), built by block diagonals (kern_trigMat_inv) */
    double *X = (double *)calloc((size_t)n * n, sizeof(double));
    for (int j = 0; j < nb; ++j)
        for (int u = 0; u < 3; ++u)
            for (int v = 0; v < 3; ++v) X[(size_t)(j * 3 + u) * n + j * 3 + v] = dinv[9 * j + u * 3 + v];
    for (int ii = 1; ii < nb; ++ii) {
#pragma omp parallel for schedule(static)
        for (int j = 0; j < nb - ii; ++j) {
            int i = j + ii;
            double Tb[9];
            for (int u = 0; u < 3; ++u)
                for (int v = 0; v < 3; ++v) {
                    double tt = 0.0;
                    for (int k = j; k < i; ++k) {
                        const double *l = S + (size_t)(i * 3 + u) * n + k * 3;
                        tt += l[0] * X[(size_t)(k * 3 + 0) * n + j * 3 + v];
                        tt += l[1] * X[(size_t)(k * 3 + 1) * n + j * 3 + v];
                        tt += l[2] * X[(size_t)(k * 3 + 2) * n + j * 3 + v];
                    }
                    Tb[u * 3 + v] = tt;
                }
            const double *Li = dinv + 9 * (size_t)i;
            for (int u = 0; u < 3; ++u)
                for (int v = 0; v < 3; ++v) {
                    double tt = 0.0;
                    tt += Li[u * 3 + 0] * Tb[0 * 3 + v];
                    tt += Li[u * 3 + 1] * Tb[1 * 3 + v];
                    tt += Li[u * 3 + 2] * Tb[2 * 3 + v];
                    X[(size_t)(i * 3 + u) * n + j * 3 + v] = -tt;
                }
        }
    }
    /* S^-1[u][v] = sum_{k>=u} X[k][u] X[k][v], u >= v (kern_trigMat_mul), then mirror (kern_fill_rest) */
#pragma omp parallel for schedule(dynamic, 4)
    for (int u = 0; u < n; ++u)
        for (int v = 0; v <= u; ++v) {
            double val = 0;
            for (int k = u; k < n; ++k) val += X[(size_t)k * n + u] * X[(size_t)k * n + v];
            S[(size_t)u * n + v] = val;
        }
    for (int u = 0; u < n; ++u)
        for (int v = 0; v < u; ++v) S[(size_t)v * n + u] = S[(size_t)u * n + v];
    free(X);
    free(dinv);
    return 0;
}

/* kern_matVec_mul, matVec_mul.cl:12-17 */
void orc_matvec(int n, const double *M, const double *v, double *out)
{
    for (int i = 0; i < n; ++i) {
        double sum = 0;
        for (int k = 0; k < n; ++k) sum = sum + M[(size_t)i * n + k] * v[k];
        out[i] = sum;
    }
}

/* Alternative to the explicit inverse: L y = b, L^T x = y. */
void orc_chol_solve(int n, const double *L, const double *b, double *x)
{
    double *y = (double *)malloc(sizeof(double) * (size_t)n);
    for (int i = 0; i < n; ++i) {
        double s = b[i];
        for (int k = 0; k < i; ++k) s -= L[(size_t)i * n + k] * y[k];
        y[i] = s / L[(size_t)i * n + i];
    }
    for (int i = n - 1; i >= 0; --i) {
        double s = y[i];
        for (int k = i + 1; k < n; ++k) s -= L[(size_t)k * n + i] * x[k];
        x[i] = s / L[(size_t)i * n + i];
    }
    free(y);
}

/* a17/a18: eb = gb - W^T dpa (compute_eb.cl:25-39), dpb = V^-1 eb (compute_dpb.cl:19-34) */
static void eb_dpb_ix(const orc_problem *p, const orc_index *ix, const double *W,
                      const double *Vinv, const double *g, const double *dpa, double *eb, double *dpb)
{
    int nc = p->nc;
    const int cnp = cnp_of(p);
    (void)ix;
#pragma omp parallel for schedule(static)
    for (int i = 0; i < p->np; ++i) {
        double e3[3];
        for (int c = 0; c < PNP; ++c) {
            double sum = 0;
            for (int o = ix->pt_start[i]; o < ix->pt_start[i + 1]; ++o) {
                const double *Wo = W + 3 * (size_t)cnp * o;
                const double *d = dpa + cnp * (size_t)p->obs_cam[o];
                for (int k = 0; k < cnp; ++k) sum = sum + Wo[k * 3 + c] * d[k];
            }
            e3[c] = g[(size_t)nc * cnp + i * PNP + c] - sum;
            eb[i * PNP + c] = e3[c];
        }
        const double *Vi = Vinv + 9 * (size_t)i;
        for (int r = 0; r < PNP; ++r)
            dpb[i * PNP + r] = Vi[r * 3] * e3[0] + Vi[r * 3 + 1] * e3[1] + Vi[r * 3 + 2] * e3[2];
    }
}

void orc_eb_dpb(const orc_problem *p, const double *W, const double *Vinv, const double *g,
                const double *dpa, double *eb, double *dpb)
{
    orc_index ix;
    idx_build(p, &ix, 0);
    eb_dpb_ix(p, &ix, W, Vinv, g, dpa, eb, dpb);
    idx_free(&ix);
}

/* a22: J x, compute_Jmultiply.cl:28-44, emitted only for observed (point,
 * camera) pairs in observation order; the reference's dense grid adds exact
 * zeros in between, which does not change any later sum.                    */
void orc_jmultiply(const orc_problem *p, const double *JA, const double *JB, const double *x,
                   double *out)
{
    const int cnp = cnp_of(p);
    size_t ncp = (size_t)p->nc * cnp;
#pragma omp parallel for schedule(static)
    for (int o = 0; o < p->no; ++o) {
        int i = p->obs_pt[o], j = p->obs_cam[o];
        for (int k = 0; k < MNP; ++k) {
            const double *a = JA + 2 * (size_t)cnp * o + k * cnp;
            const double *b = JB + 6 * (size_t)o + k * PNP;
            const double *xa = x + (size_t)j * cnp;
            const double *xb = x + ncp + (size_t)i * PNP;
            double sum = 0;
            for (int m = 0; m < cnp; ++m) sum += a[m] * xa[m];
            sum += b[0] * xb[0];
            sum += b[1] * xb[1];
            sum += b[2] * xb[2];
            out[2 * (size_t)o + k] = sum;
        }
    }
}

/* ------------------------------------------------------------------------ */
/* a23: modified Cholesky (Gill-Murray style) of cholmod_blk.cl with the
 * bounds of get_delta_beta (cl_cholmod.cpp:109-165) and the diagonal
 * correction E_i = sum_{k<=i} L_ik^2 - A_ii (kern_cholmod_E, :830-846).
 * Block column j is first tried as a plain 3x3-block step (kern_cholmod_blk,
 * :108-282; pivots must be finite and > 0, and every entry of L_ij below
 * must be <= beta, :340-341); otherwise its three columns are redone one at
 * a time from the original values (kern_cholmod_step1..4, :446-697):
 *   d = max(|A_xx - sum L_xk^2|, delta), L_xx = sqrt(d),
 *   C_ix = A_ix - sum_k L_ik L_xk, L_ix = C_ix / L_xx,
 *   if some L_ix > beta: L_xx = max_i |C_ix| / beta and L_ix recomputed.     */
void orc_cholmod(int n, double *S, double *E)
{
    int nb = n / 3;
    /* get_delta_beta: xi = max |off-diagonal|, gamma = max |diagonal| */
    double xi = 0, gam = 0;
    for (int r = 0; r < n; ++r) {
        double mx = 0;
        for (int k = 0; k < n; ++k) {
            if (k == r) continue;
            double t1 = fabs(S[(size_t)(r > k ? r : k) * n + (r > k ? k : r)]);
            if (t1 > mx) mx = t1;
        }
        if (mx > xi) xi = mx;
    }
    for (int r = 0; r < n; ++r) {
        double t1 = fabs(S[(size_t)r * n + r]);
        if (t1 > gam) gam = t1;
    }
    double delta = 1e-15 * fmax(xi + gam, 1);
    double beta = fmax(gam, 1e-15);
    beta = fmax(beta, xi / sqrt((double)(n * n - 1)));
    beta = sqrt(beta);

    double *diag = (double *)malloc(sizeof(double) * (size_t)n);
    double *orig = (double *)malloc(sizeof(double) * (size_t)n * 3);
    double *C = (double *)malloc(sizeof(double) * (size_t)n);
    for (int r = 0; r < n; ++r) diag[r] = S[(size_t)r * n + r];

    for (int j = 0; j < nb; ++j) {
        /* keep column block j (lower part) to restore on fallback */
        for (int r = j * 3; r < n; ++r)
            for (int v = 0; v < 3; ++v) orig[(size_t)r * 3 + v] = S[(size_t)r * n + j * 3 + v];
        int fail = 0;
        double T[9], L[6], Li[9];
        for (int u = 0; u < 3; ++u)
            for (int v = 0; v < 3; ++v) {
                double sum = S[(size_t)(j * 3 + u) * n + j * 3 + v];
                if (v > u) sum = S[(size_t)(j * 3 + v) * n + j * 3 + u];
                const double *lu = S + (size_t)(j * 3 + u) * n, *lv = S + (size_t)(j * 3 + v) * n;
                for (int k = 0; k < j; ++k)
                    sum -= (lu[3 * k] * lv[3 * k] + lu[3 * k + 1] * lv[3 * k + 1] + lu[3 * k + 2] * lv[3 * k + 2]);
                T[u * 3 + v] = sum;
            }
        /* pivots: finite and > 0 (cholmod_blk.cl:135-191) */
        {
            double p0 = T[0];
            double p1 = T[4] - T[3] * T[3] / T[0];
            double t1 = -T[8] * T[3] * T[3], t2 = 2 * T[7] * T[3] * T[6], t3 = -T[4] * T[6] * T[6];
            double t4 = T[0] * (T[4] * T[8] - T[7] * T[7]), t5 = -T[3] * T[3] + T[0] * T[4];
            double p2 = (t1 + t2 + t3 + t4) / t5;
            if (!isfinite(p0) || p0 <= 0 || !isfinite(p1) || p1 <= 0 || !isfinite(p2) || p2 <= 0) fail = 1;
            if (!fail) {
                L[0] = sqrt(p0);
                L[1] = T[3] / sqrt(T[0]);
                L[2] = sqrt(p1);
                L[3] = T[6] / sqrt(T[0]);
                L[4] = sqrt(T[0] / (T[0] * T[4] - T[3] * T[3])) * (T[7] - T[3] * T[6] / T[0]);
                L[5] = sqrt(p2);
                if (!isfinite(L[1]) || !isfinite(L[3]) || !isfinite(L[4])) fail = 1;
            }
        }
        if (!fail) {
            Li[0] = 1 / L[0]; Li[1] = 0; Li[2] = 0;
            Li[3] = -L[1] / (L[0] * L[2]); Li[4] = 1 / L[2]; Li[5] = 0;
            Li[6] = (L[1] * L[4] - L[2] * L[3]) / (L[0] * L[2] * L[5]);
            Li[7] = -L[4] / (L[2] * L[5]); Li[8] = 1 / L[5];
            double *d = S + (size_t)(j * 3) * n + j * 3;
            d[0] = L[0]; d[1] = 0; d[2] = 0;
            d[n] = L[1]; d[n + 1] = L[2]; d[n + 2] = 0;
            d[2 * n] = L[3]; d[2 * n + 1] = L[4]; d[2 * n + 2] = L[5];
            /* kern_cholmod_blk_step2 for the blocks below */
            for (int i = j + 1; i < nb; ++i) {
                double Tij[9];
                for (int u = 0; u < 3; ++u)
                    for (int v = 0; v < 3; ++v) {
                        double sum = S[(size_t)(i * 3 + u) * n + j * 3 + v];
                        const double *lu = S + (size_t)(i * 3 + u) * n, *lv = S + (size_t)(j * 3 + v) * n;
                        for (int k = 0; k < j; ++k)
                            sum -= (lu[3 * k] * lv[3 * k] + lu[3 * k + 1] * lv[3 * k + 1] + lu[3 * k + 2] * lv[3 * k + 2]);
                        Tij[u * 3 + v] = sum;
                    }
                for (int u = 0; u < 3; ++u)
                    for (int v = 0; v < 3; ++v) {
                        double sum = (Tij[u * 3] * Li[v * 3] + Tij[u * 3 + 1] * Li[v * 3 + 1] + Tij[u * 3 + 2] * Li[v * 3 + 2]);
                        S[(size_t)(i * 3 + u) * n + j * 3 + v] = sum;
                        S[(size_t)(j * 3 + v) * n + i * 3 + u] = 0;
                        if (sum > beta) fail = 1;
                    }
            }
        }
        if (!fail) continue;
        /* restore column block j and redo its three columns one at a time */
        for (int r = j * 3; r < n; ++r)
            for (int v = 0; v < 3; ++v) S[(size_t)r * n + j * 3 + v] = orig[(size_t)r * 3 + v];
        for (int col = 0; col < 3; ++col) {
            int x = j * 3 + col;
            double sum = S[(size_t)x * n + x];
            for (int k = 0; k < x; ++k) {
                double l = S[(size_t)x * n + k];
                sum -= l * l;
            }
            sum = fabs(sum);
            double dj = fmax(sum, delta);
            S[(size_t)x * n + x] = sqrt(dj);
            int big = 0;
            for (int i = x + 1; i < n; ++i) {
                double c = S[(size_t)i * n + x];
                for (int k = 0; k < x; ++k) c = c - (S[(size_t)i * n + k] * S[(size_t)x * n + k]);
                C[i] = c;
                double l = c / S[(size_t)x * n + x];
                S[(size_t)i * n + x] = l;
                S[(size_t)x * n + i] = 0;
                if (l > beta) big = 1;
            }
            if (big) {
                double theta = 0.0;
                for (int i = x + 1; i < n; ++i) theta = fmax(theta, fabs(C[i]));
                S[(size_t)x * n + x] = theta / beta;
                for (int i = x + 1; i < n; ++i) S[(size_t)i * n + x] = C[i] / S[(size_t)x * n + x];
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        double sum = 0.0;
        for (int k = 0; k <= i; ++k) sum += S[(size_t)i * n + k] * S[(size_t)i * n + k];
        E[i] = sum - diag[i];
    }
    free(diag);
    free(orig);
    free(C);
}

/* ------------------------------------------------------------------------ */
/* drivers */

typedef struct {
    const orc_problem *p;
    orc_index ix;
    int nc, np, no, cnp, ncp, ntot;
    double *ex, *JA, *JB, *U, *V, *W, *g, *UVdiag, *Vinv, *Y, *S, *Saux, *ea, *dp, *eb;
    double *ncams, *npts, *Jx1, *Jx2, *PU, *PB, *P, *E, *tmpn;
} orc_ws;

static void ws_init(orc_ws *w, const orc_problem *p)
{
    memset(w, 0, sizeof(*w));
    w->p = p;
    w->nc = p->nc;
    w->np = p->np;
    w->no = p->no;
    w->cnp = cnp_of(p);
    w->ncp = p->nc * w->cnp;
    w->ntot = w->ncp + p->np * PNP;
    idx_build(p, &w->ix, 1);
    size_t no = (size_t)p->no, nt = (size_t)w->ntot, N = (size_t)w->ncp;
    w->ex = malloc(sizeof(double) * 2 * no + 8);
    w->JA = malloc(sizeof(double) * 2 * w->cnp * no + 8);
    w->JB = malloc(sizeof(double) * 6 * no + 8);
    w->U = malloc(sizeof(double) * w->cnp * w->cnp * (size_t)p->nc + 8);
    w->V = malloc(sizeof(double) * 9 * (size_t)p->np + 8);
    w->W = malloc(sizeof(double) * 3 * w->cnp * no + 8);
    w->Y = malloc(sizeof(double) * 3 * w->cnp * no + 8);
    w->g = malloc(sizeof(double) * nt + 8);
    w->UVdiag = malloc(sizeof(double) * nt + 8);
    w->Vinv = malloc(sizeof(double) * 9 * (size_t)p->np + 8);
    w->S = calloc(N * N + 1, sizeof(double));
    w->Saux = calloc(N * N + 1, sizeof(double));
    w->ea = malloc(sizeof(double) * N + 8);
    w->dp = malloc(sizeof(double) * nt + 8);
    w->eb = malloc(sizeof(double) * 3 * (size_t)p->np + 8);
    w->ncams = malloc(sizeof(double) * N + 8);
    w->npts = malloc(sizeof(double) * 3 * (size_t)p->np + 8);
    w->Jx1 = malloc(sizeof(double) * 2 * no + 8);
    w->Jx2 = malloc(sizeof(double) * 2 * no + 8);
    w->PU = malloc(sizeof(double) * nt + 8);
    w->PB = malloc(sizeof(double) * nt + 8);
    w->P = malloc(sizeof(double) * nt + 8);
    w->E = malloc(sizeof(double) * N + 8);
    w->tmpn = malloc(sizeof(double) * nt + 8);
}

static void ws_free(orc_ws *w)
{
    idx_free(&w->ix);
    double **b[] = {&w->ex, &w->JA, &w->JB, &w->U, &w->V, &w->W, &w->g, &w->UVdiag, &w->Vinv,
                    &w->Y, &w->S, &w->Saux, &w->ea, &w->dp, &w->eb, &w->ncams, &w->npts,
                    &w->Jx1, &w->Jx2, &w->PU, &w->PB, &w->P, &w->E, &w->tmpn};
    for (size_t k = 0; k < sizeof(b) / sizeof(b[0]); ++k) {
        free(*b[k]);
        *b[k] = NULL;
    }
}

static void trace_push(orc_result *res, int itno, int kind, int acc, double damping, double rho,
                       double cost, double lambda)
{
    if (!res || !res->trace || res->n_trace >= res->trace_cap) {
        if (res) res->n_trace++;
        return;
    }
    orc_trace *t = &res->trace[res->n_trace++];
    t->itno = itno;
    t->kind = kind;
    t->accepted = acc;
    t->pad = 0;
    t->damping = damping;
    t->rho = rho;
    t->cost = cost;
    t->lambda = lambda;
}

/* Reduced-camera solve for the current S (lower) and ea: dpa.  Returns 0 if
 * S was factored.  solve_mode 0: S^-1 then S^-1 ea (SPDinv + matVec_mul);
 * solve_mode 1: Cholesky + two triangular solves.                            */
static int reduced_solve(orc_ws *w, int mode, double *dpa)
{
    int N = w->ncp;
    if (N % 3 != 0) {  /* variable intrinsics: no 3x3-block form; column Cholesky + solves */
        if (col_cholesky(N, w->S)) return 1;
        orc_chol_solve(N, w->S, w->ea, dpa);
        return 0;
    }
    if (mode == 0) {
        if (orc_spd_inverse(N, w->S)) return 1;
        orc_matvec(N, w->S, w->ea, dpa);
        return 0;
    }
    if (orc_cholesky(N, w->S)) return 1;
    orc_chol_solve(N, w->S, w->ea, dpa);
    return 0;
}

static void newp(orc_ws *w, const double *cams, const double *pts, const double *dp)
{
    for (int k = 0; k < w->ncp; ++k) w->ncams[k] = cams[k] + dp[k];
    for (int k = 0; k < w->np * PNP; ++k) w->npts[k] = pts[k] + dp[w->ncp + k];
}

/* levmar(), levmar.cpp:45-256 */
static int levmar_ws(orc_ws *w, double *cams, double *pts, const orc_opts *o, int *itno,
                     orc_result *res)
{
    const orc_problem *p = w->p;
    int nt = w->ntot, ncp = w->ncp;
    double tau = o->tau, mu = 0, rho, p_L2 = 0, dp_L2, ex_L2, new_ex_L2;
    int nu = 2, gooditer_cnt = 0, first = 1;
    int iter_flag;

    orc_residual(p, cams, pts, w->ex);
    ex_L2 = orc_sumsq(2 * w->no, w->ex);
    if (res) res->initial_cost = ex_L2;

    iter_flag = ORC_ITER_CONTINUE;
    for (; *itno < o->max_iter && iter_flag == ORC_ITER_CONTINUE; (*itno)++) {
        orc_jacobian(p, cams, pts, w->JA, w->JB);
        normal_blocks_ix(p, &w->ix, w->JA, w->JB, w->ex, 1.0, w->U, w->V, w->W, w->g, w->UVdiag);
        if (first) { /* levmar.cpp:114-120, maxElmOfUV sba_func.cpp:422-444 */
            double mx = 0.0;
            for (int k = 0; k < nt; ++k)
                if (w->UVdiag[k] > mx) mx = w->UVdiag[k];
            mu = tau * mx;
            first = 0;
            p_L2 = 1e+3;
            nu = 2;
        }
        while (1) {
            orc_vinv(w->np, w->V, mu, w->Vinv);
            orc_yblocks(p, w->W, w->Vinv, w->Y);
            schur_ix(p, &w->ix, w->U, mu, w->Y, w->W, w->S);
            ea_ix(p, &w->ix, w->Y, w->g, w->ea);
            if (reduced_solve(w, o->solve_mode, w->dp) == 0) {
                eb_dpb_ix(p, &w->ix, w->W, w->Vinv, w->g, w->dp, w->eb, w->dp + ncp);
                dp_L2 = orc_sumsq(nt, w->dp);
                if (dp_L2 < p_L2 * o->stop_thresh * o->stop_thresh) {
                    iter_flag = ORC_ITER_DP_NO_CHANGE;
                    trace_push(res, *itno, ORC_TR_LM_STOP, 0, mu, NAN, NAN, 0);
                    break;
                }
                if (dp_L2 >= (p_L2 + o->stop_thresh) / (o->eps * o->eps)) {
                    iter_flag = ORC_ITER_ERR;
                    trace_push(res, *itno, ORC_TR_LM_STOP, 0, mu, NAN, NAN, 0);
                    break;
                }
                newp(w, cams, pts, w->dp);
                orc_residual(p, w->ncams, w->npts, w->ex);
                new_ex_L2 = orc_sumsq(2 * w->no, w->ex);
                { /* compute_rho, levmar.cpp:271-280 */
                    double sum = 0;
                    for (int i = 0; i < nt; ++i) sum += w->dp[i] * (mu * w->dp[i] + w->g[i]);
                    rho = (ex_L2 - new_ex_L2) / sum;
                }
                if (rho > 0) {
                    double mu_used = mu;
                    double tmp = 2 * rho - 1;
                    tmp = 1.0 - tmp * tmp * tmp;
                    mu = mu * ((tmp >= (1.0 / 3.0)) ? tmp : (1.0 / 3.0));
                    nu = 2;
                    memcpy(cams, w->ncams, sizeof(double) * (size_t)ncp);
                    memcpy(pts, w->npts, sizeof(double) * (size_t)w->np * PNP);
                    p_L2 = orc_sumsq(ncp, cams);
                    {
                        double s2 = p_L2;
                        for (int k = 0; k < w->np * PNP; ++k) s2 += pts[k] * pts[k];
                        p_L2 = s2;
                    }
                    ex_L2 = new_ex_L2;
                    trace_push(res, *itno, ORC_TR_LM_TRIAL, 1, mu_used, rho, new_ex_L2, 0);
                    if (fabs(rho - 1) < (1.0 / 5.0)) {
                        gooditer_cnt++;
                        if (gooditer_cnt >= 5 && o->allow_switch) {
                            iter_flag = ORC_ITER_TURN_TO_TR;
                            break;
                        }
                    } else
                        gooditer_cnt = 0;
                    break;
                }
                trace_push(res, *itno, ORC_TR_LM_TRIAL, 0, mu, rho, new_ex_L2, 0);
            } else {
                gooditer_cnt = 0;
                trace_push(res, *itno, ORC_TR_LM_SOLVE_FAIL, 0, mu, NAN, NAN, 0);
            }
            mu *= nu;
            {
                /* levmar.cpp:238-243: nu is an int; 2*nu wraps at 2^31 */
                int nu2 = (int)(2u * (unsigned)nu);
                if (nu2 <= nu) {
                    iter_flag = ORC_ITER_ERR;
                    break;
                }
                nu = nu2;
            }
        }
        if (ex_L2 <= o->stop_thresh) iter_flag = ORC_ITER_ERR_SMALL_ENOUGH;
    }
    if (res) {
        res->final_cost = ex_L2;
        res->status = iter_flag;
        res->iterations = *itno;
    }
    return iter_flag;
}

/* compute_PB, trust_region.cpp:292-405 */
static int compute_pb(orc_ws *w, const orc_opts *o, double *lambda)
{
    const orc_problem *p = w->p;
    int N = w->ncp;
    orc_vinv(w->np, w->V, *lambda, w->Vinv);
    orc_yblocks(p, w->W, w->Vinv, w->Y);
    schur_ix(p, &w->ix, w->U, *lambda, w->Y, w->W, w->S);
    memcpy(w->Saux, w->S, sizeof(double) * (size_t)N * N);
    ea_ix(p, &w->ix, w->Y, w->g, w->ea);
    if (reduced_solve(w, o->solve_mode, w->dp)) {
        if (*lambda == 0.0) {
            double sum = 0.0;
            if (N % 3 == 0) {
                memcpy(w->S, w->Saux, sizeof(double) * (size_t)N * N);
                orc_cholmod(N, w->S, w->E);
                for (int i = 0; i < N; ++i) sum += w->E[i];
            } else {
                /* 11/16-parameter cameras (no reference counterpart): the
                 * 3x3-block modified Cholesky on S padded to a multiple of 3
                 * with an identity block; lambda from the first N corrections */
                const int n3 = N + (3 - N % 3);
                double *Sp = (double *)calloc((size_t)n3 * n3, sizeof(double));
                double *Ep = (double *)malloc(sizeof(double) * (size_t)n3);
                for (int r = 0; r < N; ++r) memcpy(Sp + (size_t)r * n3, w->Saux + (size_t)r * N, sizeof(double) * N);
                for (int r = N; r < n3; ++r) Sp[(size_t)r * n3 + r] = 1.0;
                orc_cholmod(n3, Sp, Ep);
                for (int i = 0; i < N; ++i) sum += Ep[i];
                free(Sp);
                free(Ep);
            }
            *lambda = fabs(sum) / N;
            return 0;
        }
        *lambda = 2 * (*lambda);
        return 0;
    }
    eb_dpb_ix(p, &w->ix, w->W, w->Vinv, w->g, w->dp, w->eb, w->dp + N);
    for (int i = 0; i < w->ntot; ++i) w->PB[i] = -w->dp[i];
    return 1;
}

/* compute_p_2, trust_region.cpp:520-595 (2-D subspace step, else dogleg) */
static double compute_p2(int n, double a, double b, double c, double delta, const double *PU,
                         const double *PB, double *P, const double *g)
{
    double pUg = dotp(n, PU, g), pBg = dotp(n, PB, g);
    double eta1 = (pBg * b) / (-b * b + c * a) - (c * pUg) / (-b * b + c * a);
    double eta2 = (pUg * b) / (-b * b + c * a) - (pBg * a) / (-b * b + c * a);
    double p_norm = 0.0;
    for (int i = 0; i < n; ++i) {
        P[i] = eta1 * PU[i] + eta2 * PB[i];
        p_norm += P[i] * P[i];
    }
    p_norm = sqrt(p_norm);
    if (p_norm > delta) {
        double pU_norm = 0.0, pB_norm = 0.0;
        for (int i = 0; i < n; ++i) {
            pU_norm += PU[i] * PU[i];
            pB_norm += PB[i] * PB[i];
        }
        pU_norm = sqrt(pU_norm);
        pB_norm = sqrt(pB_norm);
        if (pU_norm > delta) {
            for (int i = 0; i < n; ++i) P[i] = delta * PU[i] / pU_norm;
            return delta;
        } else if (pB_norm <= delta) {
            for (int i = 0; i < n; ++i) {
                P[i] = PB[i];
                p_norm += P[i] * P[i]; /* not reset, as trust_region.cpp:564-569 */
            }
            return sqrt(p_norm);
        } else {
            double A = 0.0, B = 0.0, Cc = 0.0, Ai, Bi, d2, tau;
            for (int i = 0; i < n; ++i) {
                Ai = PB[i] - PU[i];
                Bi = 2 * PU[i] - PB[i];
                A += Ai * Ai;
                B += Ai * Bi;
                Cc += Bi * Bi;
            }
            B = 2 * B;
            Cc = Cc - delta * delta;
            d2 = B * B - 4 * A * Cc;
            if (fabs(d2) < 1e-12) d2 = 0;
            tau = (-B + sqrt(d2)) / (2 * A);
            for (int i = 0; i < n; ++i) P[i] = PU[i] + (tau - 1) * (PB[i] - PU[i]);
            return delta;
        }
    }
    return p_norm;
}

/* trust_region(), trust_region.cpp:49-288 */
static int trust_region_ws(orc_ws *w, double *cams, double *pts, const orc_opts *o, int *itno,
                           orc_result *res)
{
    const orc_problem *p = w->p;
    int nt = w->ntot, ncp = w->ncp, no2 = 2 * w->no;
    int iter_flag = ORC_ITER_CONTINUE, notgood_cnt = 0, good_iters = 0, nu = 2;
    double ex_L2, act_ex_L2, pred_ex_L2, gtBg, gtg, dk = 1, lambda = 0, origin_lambda = 0.0;

    orc_residual(p, cams, pts, w->ex);
    ex_L2 = orc_sumsq(no2, w->ex);
    if (res && res->n_trace == 0) res->initial_cost = ex_L2;
    double final_err = ex_L2; /* *finalErr of trust_region.cpp: set on every accepted step */

    for (; *itno < o->max_iter; (*itno)++) {
        orc_jacobian(p, cams, pts, w->JA, w->JB);
        /* g = -2 J^T e (compute_g with coeff -2), U, V, W with coeff 2 */
        normal_blocks_ix(p, &w->ix, w->JA, w->JB, w->ex, -2.0, w->U, w->V, w->W, w->g, w->UVdiag);
        /* the U/V/W of coeff 2 are the negatives of coeff -2 */
        for (int k = 0; k < w->cnp * w->cnp * w->nc; ++k) w->U[k] = -w->U[k];
        for (int k = 0; k < 9 * w->np; ++k) w->V[k] = -w->V[k];
        for (long long k = 0; k < 3LL * w->cnp * w->no; ++k) w->W[k] = -w->W[k];
        for (int k = 0; k < nt; ++k) w->UVdiag[k] = -w->UVdiag[k];
        orc_jmultiply(p, w->JA, w->JB, w->g, w->Jx1);
        gtBg = 2 * dotp(no2, w->Jx1, w->Jx1);
        gtg = dotp(nt, w->g, w->g);
        for (int i = 0; i < nt; ++i) w->PU[i] = -(w->g[i] * gtg) / gtBg;

        int solved = 0;
        while (!solved) {
            double lam_used = lambda;
            solved = compute_pb(w, o, &lambda);
            if (!solved) {
                trace_push(res, *itno, ORC_TR_TR_PB_FAIL, 0, dk, NAN, NAN, lam_used);
                if (origin_lambda != 0.0) {
                    if (nu > 4) {
                        if (res) {
                            res->final_cost = final_err;
                            res->status = ORC_ITER_TURN_TO_LM;
                            res->iterations = *itno;
                        }
                        return ORC_ITER_TURN_TO_LM;
                    }
                    lambda = lambda * nu;
                    nu = nu * 2;
                }
            } else {
                nu = 2;
                origin_lambda = lambda;
            }
        }
        orc_jmultiply(p, w->JA, w->JB, w->PU, w->Jx1);
        orc_jmultiply(p, w->JA, w->JB, w->PB, w->Jx2);
        double pUtBpU = 2 * dotp(no2, w->Jx1, w->Jx1);
        double pUtBpB = 2 * dotp(no2, w->Jx1, w->Jx2);
        double pBtBpB = 2 * dotp(no2, w->Jx2, w->Jx2);

        iter_flag = ORC_ITER_CONTINUE;
        while (iter_flag == ORC_ITER_CONTINUE) {
            double dk_used = dk;
            compute_p2(nt, pUtBpU, pUtBpB, pBtBpB, dk, w->PU, w->PB, w->P, w->g);
            newp(w, cams, pts, w->P);
            orc_residual(p, w->ncams, w->npts, w->ex);
            act_ex_L2 = orc_sumsq(no2, w->ex);
            if (fabs((ex_L2 - act_ex_L2) / ex_L2) < o->eps2) {
                iter_flag = ORC_ITER_DP_NO_CHANGE;
                trace_push(res, *itno, ORC_TR_TR_TRIAL, 0, dk_used, NAN, act_ex_L2, lambda);
                break;
            }
            orc_jmultiply(p, w->JA, w->JB, w->P, w->Jx1);
            double Jx_norm = 2 * orc_sumsq(no2, w->Jx1);
            pred_ex_L2 = dotp(nt, w->g, w->P);
            pred_ex_L2 += ex_L2 + Jx_norm / 2;
            double rho = (ex_L2 - act_ex_L2) / (ex_L2 - pred_ex_L2);
            int acc = 0;
            if (rho < (1.0 / 4.0) || act_ex_L2 > ex_L2) {
                dk = dk / 4;
            } else if (rho >= (3.0 / 4.0) && act_ex_L2 < ex_L2) {
                iter_flag = ORC_ITER_PASS;
                acc = 1;
                dk = fmin(2 * dk, 10000);
            } else if (rho >= (1.0 / 4.0) && rho < (3.0 / 4.0) && act_ex_L2 < ex_L2) {
                iter_flag = ORC_ITER_PASS;
                acc = 1;
            } else if (isnan(rho)) {
                trace_push(res, *itno, ORC_TR_TR_TRIAL, 0, dk_used, rho, act_ex_L2, lambda);
                if (res) {
                    res->final_cost = ex_L2;
                    res->status = ORC_ITER_TURN_TO_LM;
                    res->iterations = *itno;
                }
                return ORC_ITER_TURN_TO_LM;
            }
            if (acc) {
                final_err = act_ex_L2;
                memcpy(cams, w->ncams, sizeof(double) * (size_t)ncp);
                memcpy(pts, w->npts, sizeof(double) * (size_t)w->np * PNP);
            }
            trace_push(res, *itno, ORC_TR_TR_TRIAL, acc, dk_used, rho, act_ex_L2, lambda);
            if (fabs((act_ex_L2 - ex_L2) / ex_L2) <= o->eps2) {
                iter_flag = ORC_ITER_ERR_SMALL_ENOUGH;
                break;
            }
            if (rho < 1.0 / 4) {
                notgood_cnt++;
                if (notgood_cnt >= 5) {
                    iter_flag = ORC_ITER_TURN_TO_LM;
                    break;
                }
            } else
                notgood_cnt = 0;
            if (rho > 3.0 / 4 && act_ex_L2 < ex_L2) {
                good_iters++;
                if (good_iters >= 10) {
                    lambda = 0.0;
                    origin_lambda = 0.0;
                    good_iters = 0;
                }
            } else
                good_iters = 0;
            if (rho > (1.0 / 4) && act_ex_L2 < ex_L2) ex_L2 = act_ex_L2;
        }
        if (iter_flag != ORC_ITER_PASS) break;
    }
    if (res) {
        res->final_cost = final_err;
        res->status = iter_flag;
        res->iterations = *itno;
    }
    return iter_flag;
}

static void set_threads(const orc_opts *o)
{
#ifdef _OPENMP
    omp_set_num_threads(o->n_threads > 0 ? o->n_threads : 1);
#else
    (void)o;
#endif
}

int orc_levmar(const orc_problem *p, double *cams, double *pts, const orc_opts *o, int *itno,
               orc_result *res)
{
    orc_ws w;
    set_threads(o);
    ws_init(&w, p);
    int r = levmar_ws(&w, cams, pts, o, itno, res);
    ws_free(&w);
    return r;
}

int orc_trust_region(const orc_problem *p, double *cams, double *pts, const orc_opts *o, int *itno,
                     orc_result *res)
{
    orc_ws w;
    set_threads(o);
    ws_init(&w, p);
    int r = trust_region_ws(&w, cams, pts, o, itno, res);
    ws_free(&w);
    return r;
}

/* main() loop, main.cpp:193-208: LM until it hands over, TR until it hands back. */
int orc_solve_hybrid(const orc_problem *p, double *cams, double *pts, const orc_opts *o,
                     orc_result *res)
{
    orc_ws w;
    int itno = 0, flag;
    double init = NAN;
    set_threads(o);
    ws_init(&w, p);
    while (1) {
        flag = levmar_ws(&w, cams, pts, o, &itno, res);
        if (res && isnan(init)) init = res->initial_cost;
        if (flag != ORC_ITER_TURN_TO_TR) break;
        flag = trust_region_ws(&w, cams, pts, o, &itno, res);
        if (flag != ORC_ITER_TURN_TO_LM) break;
    }
    if (res) res->initial_cost = init;
    ws_free(&w);
    return flag;
}

/* A problem with its index lists and work buffers built once, for timing
 * repeated driver calls (the reference builds its index tables once too,
 * PSBA/main.cpp:183-189). */
struct orc_session {
    orc_ws w;
};

orc_session *orc_session_new(const orc_problem *p)
{
    orc_session *s = (orc_session *)calloc(1, sizeof(orc_session));
    if (s) ws_init(&s->w, p);
    return s;
}

int orc_session_levmar(orc_session *s, double *cams, double *pts, const orc_opts *o, int *itno,
                       orc_result *res)
{
    set_threads(o);
    return levmar_ws(&s->w, cams, pts, o, itno, res);
}

int orc_session_trust_region(orc_session *s, double *cams, double *pts, const orc_opts *o, int *itno,
                             orc_result *res)
{
    set_threads(o);
    return trust_region_ws(&s->w, cams, pts, o, itno, res);
}

void orc_session_free(orc_session *s)
{
    if (!s) return;
    ws_free(&s->w);
    free(s);
}

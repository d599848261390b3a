/*
 * Reference kernels, run on the CPU.  TEST INFRASTRUCTURE ONLY.
 *
 * This translation unit compiles the reference's own barrier-free OpenCL C
 * kernels (CL_files/compute_*.cl, update_*.cl, restore_UVdiag.cl,
 * matVec_mul.cl) unmodified, as C++, by supplying the handful of OpenCL
 * built-ins they use (get_global_id, double3, dot) and then executing each
 * NDRange as a sequential loop over global ids.  None of these kernels uses
 * local memory, barriers or device-side enqueue, so a sequential sweep over
 * the work-items is the NDRange semantics exactly.
 *
 * Kernels that need work-group barriers or device-side enqueue (SPD_inv.cl,
 * cholmod_blk.cl) cannot be compiled this way; the oracle restates them.
 *
 * The reference sources are #included from where they lie (the include path
 * is given by oracle/build.py); nothing is copied into this repository.
 * The built library lands in oracle/_ref/ and is only used to pin the oracle
 * (oracle/psba_oracle.c) and to generate tests/golden fixtures.
 */
#include <cmath>
#include <cstdio>
#include <cstddef>

static size_t g_gid[3];
static inline size_t get_global_id(int d) { return g_gid[d]; }

struct ocl_double3 { double x, y, z; };
static inline double dot(ocl_double3 a, ocl_double3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }

#define __kernel static
#define __global
#define __local
#define dtype double
#define dtype3 ocl_double3
#define cnp 6
#define pnp 3
#define mnp 2

/* Same inclusion order as CL_files/PSBA.cl:10-38, minus the files that need
 * barriers / device-side enqueue and the never-launched compute_Bg.cl. */
#include "compute_exQT.cl"
#include "compute_jacobiQT.cl"
#include "compute_U.cl"
#include "compute_V.cl"
#include "compute_Wblks.cl"
#include "compute_g.cl"
#include "update_UV.cl"
#include "compute_Vinv.cl"
#include "restore_UVdiag.cl"
#include "compute_Yblks.cl"
#include "compute_S.cl"
#include "compute_ea.cl"
#include "matVec_mul.cl"
#include "compute_eb.cl"
#include "compute_dpb.cl"
#include "compute_newp.cl"
#include "update_p.cl"
#include "compute_Jmultiply.cl"

#undef QtX
#undef QtY
#undef QtZ
#undef X
#undef Y
#undef Z
#undef ax
#undef ay
#undef x0
#undef y0
#undef cnp
#undef pnp
#undef mnp
#undef dtype
#undef dtype3

/* Globals the reference CPU file (PSBA/levmar_func_cpu.cpp) refers to. */
FILE *debug_file = nullptr;
int itno = 0;

/* C++-linkage functions from PSBA/levmar_func_cpu.cpp (compiled alongside). */
void calcImgProjJacRTS(double a[5], double qr0[4], double v[3], double t[3],
                       double M[3], double jacmRT[2][6], double jacmS[2][3]);
void calcImgProjFullR(double a[5], double qr0[4], double t[3], double M[3], double n[2]);
void compute_proj_err(int cnp, int pnp, int mnp, int n3Dpts, int nCams, int n2Dprojs,
                      double *K, double *impts_data, double *initcams_data, double *motion_data,
                      int *iidx, int *jidx, double *ex);

static void sweep1(size_t n0) { (void)n0; }

extern "C" {

/* ---- one entry per reference kernel: NDRange as the host wrapper launches it ---- */

/* sba_func.cpp:115  global {n2Dprojs} */
void ref_compute_exQT(int nobs, double *K, double *impts, double *initcams, double *cams,
                      double *pts, int *iidx, int *jidx, double *ex) {
    for (size_t a = 0; a < (size_t)nobs; ++a) {
        g_gid[0] = a;
        kern_compute_exQT(K, impts, initcams, cams, pts, iidx, jidx, ex);
    }
}

/* sba_func.cpp:187  global {n2Dprojs} */
void ref_compute_jacobiQT(int nobs, double *K, double *impts, double *initcams, double *cams,
                          double *pts, int *iidx, int *jidx, double *JA, double *JB) {
    for (size_t a = 0; a < (size_t)nobs; ++a) {
        g_gid[0] = a;
        kern_compute_jacobiQT(K, impts, initcams, cams, pts, iidx, jidx, JA, JB);
    }
}

/* sba_func.cpp:283  global {cnp, nCams*cnp} */
void ref_compute_U(int nCams, int nPts, int nobs, double *JA, int *blk_idx, double *U,
                   double *UVdiag, double coeff) {
    for (size_t b = 0; b < (size_t)nCams * 6; ++b)
        for (size_t a = 0; a < 6; ++a) {
            g_gid[0] = a; g_gid[1] = b;
            kern_compute_U(nCams, nPts, nobs, JA, blk_idx, U, UVdiag, coeff);
        }
}

/* sba_func.cpp:369  global {pnp, n3Dpts*pnp} */
void ref_compute_V(int nCams, int nPts, int nobs, double *JB, int *blk_idx, double *V,
                   double *UVdiag, double coeff) {
    for (size_t b = 0; b < (size_t)nPts * 3; ++b)
        for (size_t a = 0; a < 3; ++a) {
            g_gid[0] = a; g_gid[1] = b;
            kern_compute_V(nCams, nPts, nobs, JB, blk_idx, V, UVdiag, coeff);
        }
}

/* sba_func.cpp:485  global {cnp, n2Dprojs*pnp} */
void ref_compute_Wblks(int nCams, int nPts, int nobs, double *JA, double *JB, int *iidx,
                       int *jidx, double *W, double coeff) {
    for (size_t b = 0; b < (size_t)nobs * 3; ++b)
        for (size_t a = 0; a < 6; ++a) {
            g_gid[0] = a; g_gid[1] = b;
            kern_compute_Wblks(nCams, nPts, nobs, JA, JB, iidx, jidx, W, coeff);
        }
}

/* sba_func.cpp:569  global {nCams*cnp + n3Dpts*pnp} */
void ref_compute_g(int nCams, int nPts, int nobs, double coeff, double *JA, double *JB,
                   int *blk_idx, double *ex, double *g) {
    for (size_t a = 0; a < (size_t)nCams * 6 + (size_t)nPts * 3; ++a) {
        g_gid[0] = a;
        kern_compute_g(nCams, nPts, nobs, coeff, JA, JB, blk_idx, ex, g);
    }
}

/* sba_func.cpp:641  global {nCams*cnp + n3Dpts*pnp} */
void ref_update_UV(int nCams, int nPts, double *U, double *V, double mu) {
    for (size_t a = 0; a < (size_t)nCams * 6 + (size_t)nPts * 3; ++a) {
        g_gid[0] = a;
        kern_update_UV(nCams, nPts, U, V, mu);
    }
}

/* sba_func.cpp:709 */
void ref_restore_UVdiag(int nCams, int nPts, double *U, double *V, double *UVdiag) {
    for (size_t a = 0; a < (size_t)nCams * 6 + (size_t)nPts * 3; ++a) {
        g_gid[0] = a;
        kern_restore_UVdiag(nCams, nPts, U, V, UVdiag);
    }
}

/* sba_func.cpp:748  global {n3Dpts} */
void ref_compute_Vinv(int nPts, double *V, double *ret) {
    for (size_t a = 0; a < (size_t)nPts; ++a) {
        g_gid[0] = a;
        kern_compute_Vinv(nPts, V, ret);
    }
}

/* sba_func.cpp:822  global {cnp, n2Dprojs*pnp} */
void ref_compute_Yblks(int nCams, int nPts, int nobs, int *iidx, double *W, double *Vinv,
                       double *Y) {
    for (size_t b = 0; b < (size_t)nobs * 3; ++b)
        for (size_t a = 0; a < 6; ++a) {
            g_gid[0] = a; g_gid[1] = b;
            kern_compute_Yblks(nCams, nPts, iidx, W, Vinv, Y);
        }
}

/* sba_func.cpp:898  global {N, N} */
void ref_compute_S(int nCams, int nPts, int *blk_idx, double *U, double *Y, double *W,
                   int *comm3DIdx, int *comm3DIdxCnt, double *S) {
    size_t N = (size_t)nCams * 6;
    for (size_t b = 0; b < N; ++b)
        for (size_t a = 0; a < N; ++a) {
            g_gid[0] = a; g_gid[1] = b;
            kern_compute_S(nCams, nPts, blk_idx, U, Y, W, comm3DIdx, comm3DIdxCnt, S);
        }
}

/* sba_func.cpp:965  global {nCams*cnp} */
void ref_compute_ea(int nCams, int nPts, int nobs, int *blk_idx, double *Y, double *g,
                    double *ea) {
    for (size_t a = 0; a < (size_t)nCams * 6; ++a) {
        g_gid[0] = a;
        kern_compute_ea(nCams, nPts, nobs, blk_idx, Y, g, ea);
    }
}

/* cl_linearalg.cpp:31  global {dim} */
void ref_matVec_mul(int dim, double *M, double *v, double *out) {
    for (size_t a = 0; a < (size_t)dim; ++a) {
        g_gid[0] = a;
        kern_matVec_mul(dim, M, v, out);
    }
}

/* sba_func.cpp:1030  global {n3Dpts*pnp} */
void ref_compute_eb(int nCams, int nPts, int nobs, int *blk_idx, double *W, double *dp,
                    double *g, double *eab) {
    for (size_t a = 0; a < (size_t)nPts * 3; ++a) {
        g_gid[0] = a;
        kern_compute_eb(nCams, nPts, nobs, blk_idx, W, dp, g, eab);
    }
}

/* sba_func.cpp:1090  global {n3Dpts*pnp} */
void ref_compute_dpb(int nCams, int nPts, double *Vinv, double *eab, double *dp) {
    for (size_t a = 0; a < (size_t)nPts * 3; ++a) {
        g_gid[0] = a;
        kern_compute_dpb(nCams, nPts, Vinv, eab, dp);
    }
}

/* sba_func.cpp:1142 */
void ref_compute_newp(int nCamParas, int nPtParas, double *cams, double *pts, double *dp,
                      double *new_cams, double *new_pts) {
    for (size_t a = 0; a < (size_t)nCamParas + (size_t)nPtParas; ++a) {
        g_gid[0] = a;
        kern_compute_newp(nCamParas, nPtParas, cams, pts, dp, new_cams, new_pts);
    }
}

/* sba_func.cpp:45  global {nCams*n3Dpts*mnp} */
void ref_compute_Jmultiply(int nCams, int nPts, int nobs, double *JA, double *JB, int *blk_idx,
                           double *x, double *out) {
    for (size_t a = 0; a < (size_t)nCams * (size_t)nPts * 2; ++a) {
        g_gid[0] = a;
        kern_compute_Jmultiply(nCams, nPts, nobs, JA, JB, blk_idx, x, out);
    }
}

/* ---- PSBA/levmar_func_cpu.cpp ---- */
void ref_calcImgProjJacRTS(double *a, double *qr0, double *v, double *t, double *M,
                           double *jacA /*2x6*/, double *jacB /*2x3*/) {
    calcImgProjJacRTS(a, qr0, v, t, M, (double(*)[6])jacA, (double(*)[3])jacB);
}

void ref_calcImgProjFullR(double *a, double *qr0, double *t, double *M, double *n) {
    calcImgProjFullR(a, qr0, t, M, n);
}

void ref_compute_proj_err(int nPts, int nCams, int nobs, double *K, double *impts,
                          double *initcams, double *motion, int *iidx, int *jidx, double *ex) {
    compute_proj_err(6, 3, 2, nPts, nCams, nobs, K, impts, initcams, motion, iidx, jidx, ex);
}

} /* extern "C" */

/*
 * FP64 CPU oracle for the sparse bundle-adjustment LM / trust-region path.
 * TEST INFRASTRUCTURE ONLY: tests, the smoke check and the bench's CPU
 * baseline use it as the checker; the product never links it.
 *
 * It restates, in plain C, the reference's OpenCL kernel chain
 * (CL_files/compute_*.cl, SPD_inv.cl, cholmod_blk.cl, ...) and its two host
 * drivers (PSBA/levmar.cpp, PSBA/trust_region.cpp) with the reference's
 * data layouts and summation orders.  Each function cites the reference
 * file:line it follows.
 *
 * Layouts (all row-major, FP64, as the reference stores them):
 *   K      5 per camera   fx, cx, cy, aspect, skew         (psba.h:3, main.cpp:141-149)
 *   q0     4 per camera   s, v1, v2, v3 initial rotation   (readparams.cpp:223-226)
 *   cams   6 per camera   v1, v2, v3 (local quat vector part), t1, t2, t3
 *   pts    3 per point
 *   meas   2 per observation, observations sorted (point asc, camera asc)
 *   JA 2x6, JB 2x3, W/Y 6x3 per observation; U 6x6 per camera; V 3x3 per point
 *   g = [ga (6C) | gb (3P)];  S dense N x N, N = 6C (only the lower triangle is defined)
 *
 * Variable intrinsics (no counterpart in the reference, whose kernels fix
 * cnp = 6, CL_files/PSBA.cl:5): cnp = 11 appends the intrinsics in the
 * reference's K layout (fx, cx, cy, ar, skew) to each camera's 6 pose
 * parameters, cnp = 16 further appends distortion (k1, k2, p1, p2, k3) in
 * the Bouguet order of the sba camera files (data/54camsvarKD.txt); the
 * 6-wide blocks above become cnp-wide (JA 2 x cnp, W/Y cnp x 3, U cnp x cnp).
 */
#ifndef PSBA_ORACLE_H
#define PSBA_ORACLE_H
#ifdef __cplusplus
extern "C" {
#endif

/* status codes, PSBA/psba.h:12-18 */
#define ORC_ITER_TURN_TO_LM 1
#define ORC_ITER_TURN_TO_TR 2
#define ORC_ITER_CONTINUE 3
#define ORC_ITER_ERR 4
#define ORC_ITER_DP_NO_CHANGE 5
#define ORC_ITER_ERR_SMALL_ENOUGH 6
#define ORC_ITER_PASS 7

/* trace record kinds */
#define ORC_TR_LM_TRIAL 1     /* LM trial that produced a step (rho computed) */
#define ORC_TR_LM_SOLVE_FAIL 2 /* LM trial whose reduced system was not SPD */
#define ORC_TR_TR_TRIAL 3     /* dogleg trial */
#define ORC_TR_TR_PB_FAIL 4   /* trust-region Gauss-Newton step failed (lambda raised) */
#define ORC_TR_LM_STOP 5      /* LM trial stopped by the dp tests */

typedef struct {
    int itno;      /* global iteration counter when the record was made */
    int kind;      /* ORC_TR_* */
    int accepted;  /* 1 if the parameters were updated */
    int pad;
    double damping;  /* mu (LM) or trust radius before the trial (TR) */
    double rho;      /* gain ratio (NaN when not computed) */
    double cost;     /* cost at the trial point (NaN when not computed) */
    double lambda;   /* TR only: lambda used for the Gauss-Newton step */
} orc_trace;

typedef struct {
    int nc, np, no;
    const double *K;      /* 5 per camera; read only when cnp == 6 */
    const double *q0;
    const double *meas;
    const int *obs_pt;
    const int *obs_cam;
    int cnp;              /* parameters per camera: 6 (0 means 6), 11, 16 */
    const double *wt;     /* NULL, or per observation a, b, c of the upper factor
                             L = [[a, b], [0, c]] with L^T L = cov^-1: residual and
                             Jacobian rows are whitened, e <- L e, J <- L J */
} orc_problem;

typedef struct {
    double tau;          /* PSBA_INIT_MU      psba.h:6 */
    double stop_thresh;  /* PSBA_STOP_THRESH  psba.h:7 */
    double eps;          /* PSBA_EPSILON      psba.h:8 */
    double eps2;         /* PSBA_EPSILON2     psba.h:9 */
    int max_iter;        /* itno < 50         levmar.cpp:100 */
    int allow_switch;    /* 1: LM may hand over to TR and back, as the reference */
    int solve_mode;      /* 0: explicit S^-1 as SPD_inv.cl; 1: Cholesky + triangular solves */
    int n_threads;       /* OpenMP threads for the independent loops (results do not depend on it) */
} orc_opts;

typedef struct {
    int status;
    int iterations;       /* value of the global iteration counter on return */
    double initial_cost;
    double final_cost;
    int n_trace;
    int trace_cap;
    orc_trace *trace;     /* caller-owned, trace_cap entries */
} orc_result;

void orc_default_opts(orc_opts *o);

/* ---- stages (reference layouts) ---- */
void orc_residual(const orc_problem *p, const double *cams, const double *pts, double *ex);
double orc_sumsq(int n, const double *x);
void orc_jacobian(const orc_problem *p, const double *cams, const double *pts, double *JA, double *JB);
void orc_normal_blocks(const orc_problem *p, const double *JA, const double *JB, const double *ex,
                       double coeff, double *U, double *V, double *W, double *g, double *UVdiag);
void orc_vinv(int np, const double *V, double mu, double *Vinv /* 9 per point, symmetric */);
void orc_yblocks(const orc_problem *p, const double *W, const double *Vinv, double *Y);
void orc_schur(const orc_problem *p, const double *U, double mu, const double *Y, const double *W,
               double *S /* N x N, lower filled */);
void orc_ea(const orc_problem *p, const double *Y, const double *g, double *ea);
int orc_spd_inverse(int n, double *S /* in: lower; out: full inverse */);
int orc_cholesky(int n, double *S /* in: lower; out: L in lower, upper zero */);
void orc_chol_solve(int n, const double *L, const double *b, double *x);
void orc_matvec(int n, const double *M, const double *v, double *out);
void orc_eb_dpb(const orc_problem *p, const double *W, const double *Vinv, const double *g,
                const double *dpa, double *eb, double *dpb);
void orc_jmultiply(const orc_problem *p, const double *JA, const double *JB, const double *x,
                   double *out /* 2 per observation */);
void orc_cholmod(int n, double *S /* in: lower; out: modified L */, double *E);

/* ---- drivers ---- */
int orc_levmar(const orc_problem *p, double *cams, double *pts, const orc_opts *o, int *itno,
               orc_result *res);
int orc_trust_region(const orc_problem *p, double *cams, double *pts, const orc_opts *o, int *itno,
                     orc_result *res);
int orc_solve_hybrid(const orc_problem *p, double *cams, double *pts, const orc_opts *o,
                     orc_result *res);

long long orc_pair_count(const orc_problem *p);

/* problem with its index lists and buffers built once, for repeated driver calls */
typedef struct orc_session orc_session;
orc_session *orc_session_new(const orc_problem *p);
int orc_session_levmar(orc_session *s, double *cams, double *pts, const orc_opts *o, int *itno,
                       orc_result *res);
int orc_session_trust_region(orc_session *s, double *cams, double *pts, const orc_opts *o, int *itno,
                             orc_result *res);
void orc_session_free(orc_session *s);

#ifdef __cplusplus
}
#endif
#endif

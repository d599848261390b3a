// Internal declarations shared by the kernels, the dense solver and the host
// drivers.  Not part of the C ABI.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <string>
#include <vector>

#include "../../include/psba.h"

namespace psba {

// 1 / x: the hardware's approximate reciprocal (rcp.approx.ftz.f64, ~2^-20
// relative error) and one step of the order-3 Householder iteration for
// f(y) = 1/y - x: with e = 1 - x y, y <- y (1 + e + e^2), cubing the
// relative error.  Within 1 ulp of 1.0 / x for x in [2^-80, 2^80] (the dense
// factor's pivot chain; the projections' 1 / depth), in ~200 cycles and four
// FP64 instructions against ~330 cycles for the division.
#ifdef __CUDACC__
__device__ __forceinline__ double rcp_fast(double x)
{
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double e = fma(-x, y, 1.0);
    return fma(y, fma(e, e, e), y);
}

// x as two FP32 values hi + lo (x to ~2^-48): the mixed form's double-float
// sums take their FP64 operands in this form, split once where they are made
__device__ __forceinline__ float2 split2f(double x)
{
    const float hi = (float)x;
    return make_float2(hi, (float)(x - (double)hi));
}

// s + e = a + b exactly (Knuth's TwoSum), FP32
__device__ __forceinline__ void two_sum_f(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float z = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, z)), __fsub_rn(b, z));
}

// Double-float arithmetic: a value is an unevaluated sum hi + lo of two
// FP32 numbers (Dekker, "A floating-point technique for extending the
// available precision", Numer. Math. 18, 1971; Knuth's TwoSum): products
// split exactly by an FMA, sums carried with TwoSum, each result renormalised,
// ~2^-44 relative per operation.
struct df {
    float hi, lo;
};
__device__ __forceinline__ df df_of(float2 v) { return df{v.x, v.y}; }
__device__ __forceinline__ df df_renorm(float s, float e)  // |s| >= |e|
{
    const float h = __fadd_rn(s, e);
    return df{h, __fsub_rn(e, __fsub_rn(h, s))};
}
__device__ __forceinline__ df df_add(df x, df y)
{
    const float s = __fadd_rn(x.hi, y.hi), z = __fsub_rn(s, x.hi);
    const float e = __fadd_rn(__fsub_rn(x.hi, __fsub_rn(s, z)), __fsub_rn(y.hi, z));
    return df_renorm(s, e + (x.lo + y.lo));
}
__device__ __forceinline__ df df_neg(df x) { return df{-x.hi, -x.lo}; }
__device__ __forceinline__ df df_mul(df x, df y)
{
    const float p = __fmul_rn(x.hi, y.hi);
    const float e = fmaf(x.hi, y.lo, fmaf(x.lo, y.hi, fmaf(x.hi, y.hi, -p)));
    return df_renorm(p, e);
}
// 1 / x: the FP32 reciprocal, then one Newton step r + r (1 - x r) in
// double-float (doubling its ~24 correct bits)
__device__ __forceinline__ df df_rcp(df x)
{
    const float r = __frcp_rn(x.hi);
    const df xr = df_mul(x, df{r, 0.0f});
    const df e = df_add(df{1.0f, 0.0f}, df_neg(xr));
    return df_add(df{r, 0.0f}, df_mul(df{r, 0.0f}, e));
}

// w0 v0 + w1 v1 + w2 v2 with each v = hi + lo (two FP32 values), rounded
// once to FP32: the products w hi split exactly by an FMA, the w lo products
// and the errors summed beside a TwoSum chain, so the result is the FP32
// rounding of the sum computed to ~2^-44 of its terms (double-float
// arithmetic), as if formed in FP64 and rounded on store.
__device__ __forceinline__ float dot3_df(float w0, float w1, float w2, float2 v0, float2 v1, float2 v2)
{
    const float p0 = __fmul_rn(w0, v0.x), p1 = __fmul_rn(w1, v1.x), p2 = __fmul_rn(w2, v2.x);
    float lo = fmaf(w0, v0.x, -p0) + fmaf(w1, v1.x, -p1) + fmaf(w2, v2.x, -p2);
    lo = fmaf(w0, v0.y, lo);
    lo = fmaf(w1, v1.y, lo);
    lo = fmaf(w2, v2.y, lo);
    float s1, t1, s2, t2;
    two_sum_f(p0, p1, s1, t1);
    two_sum_f(s1, p2, s2, t2);
    return __fadd_rn(s2, (t1 + t2) + lo);
}
#endif

constexpr int CNP = 6;   // camera parameters (rotation vector part + translation)
constexpr int PNP = 3;   // point parameters
constexpr int MNP = 2;   // image coordinates
constexpr int CAMTAB = 56;  // doubles per camera table entry (CamTab)
constexpr int CAMTAB32 = 40;  // floats per FP32 camera table entry: M, D, fx, sk, fy (the mixed Jacobian)
constexpr int RES_TAB2F = 18;  // FP32 pairs per camera of the mixed projection: M, t, fx sk cx fy cy, a pad (16-byte rows)
constexpr int TILE = 16;    // dense Cholesky tile size
constexpr int SCHUR_CHUNK = 32;  // pair-list entries per off-diagonal Schur work unit (11/16-parameter cameras)
constexpr int OFF_MIN_LEN = 8;   // 6-parameter cameras: fewest pair-list entries per off-diagonal chunk
constexpr int MX_UNIT = 256;     // 6-parameter cameras, FP32 products: pair-list entries per warp unit
constexpr int DIAG_CHUNK = 16;   // observations per diagonal Schur work unit (11/16-parameter cameras)
constexpr int SD_THREADS = 128, SD_PER = 8;     // 6-parameter cameras: one CTA per unit, 8 observations a thread
constexpr int DIAG_SUPER = SD_THREADS * SD_PER;  // observations per diagonal unit, 6-parameter cameras
constexpr int CAM_CHUNK = 512;   // observations per camera-reduction work unit (11/16-parameter cameras)
constexpr int CAM_PER = 8, CAM_SUPER = 128 * CAM_PER;  // 6-parameter cameras: 8 observations a thread, 128 threads
// eb/dpb kernel: warps of up to EB_PPW points (in pt_order), three lanes per
// point times m = eb_lanes_per_point(views), EB_WARPS warps a block
constexpr int EB_PPW = 10, EB_WARPS = 8, EB_PPB = EB_PPW * EB_WARPS;
inline int eb_lanes_per_point(int views) { return views <= 10 ? 1 : views <= 20 ? 2 : views <= 30 ? 3 : 4; }
constexpr int RED_THREADS = 256; // threads of the reduction kernels

// Per-camera table, computed once per parameter vector on the device:
// rotation M = R(q(v) (x) q0) (row-major), the derivative of M with
// respect to each component of v (D[m]), translation and intrinsics.
struct CamTab {
    double M[9];
    double D[27];
    double t[3];
    double fx, sk, cx, fy, cy;  // fy = fx * aspect
    double ar;                  // aspect (variable intrinsics)
    double kc[5];               // k1, k2, p1, p2, k3 (16-parameter cameras; zero otherwise)
    double pad[6];
};
static_assert(sizeof(CamTab) == CAMTAB * sizeof(double), "CamTab layout");

// Scalars that one damping trial returns to the host in a single copy.
struct TrialScalars {
    double dp_L2;     // sum dp^2
    double rho_den;   // sum dp (mu dp + g)
    double new_cost;  // sum of squared residuals at p + dp
    double dot_g_dp;  // sum g dp (trust region prediction)
    int chol_status;  // 0: factored; 1: not SPD
    int pad;
    double extra[3];
};

// A unit of Schur work: a contiguous range of one camera pair's entry list
// (or of one camera's observation list for the diagonal blocks).  Units run
// in any order; `out` is the unit's position in the pair-major, chunk-ordered
// partial array that the reduction sums in order.
struct SchurUnit {
    int slot;   // camera pair (off-diagonal) or camera (diagonal)
    int begin;  // first entry
    int count;  // number of entries (<= SCHUR_CHUNK)
    int out;    // partial-sum slot
};

// Camera-reduction work unit (per-camera sums over the camera-sorted list).
struct CamUnit {
    int cam;
    int begin;
    int count;
    int pad;
};

const char *set_error(const std::string &msg);
void note_launch(int n);     // counts kernel launches (psba_kernel_launches)
long long launch_count();

// ---- kernel launchers (psba_kernels.cu) ---------------------------------

// Polls per device-side wait before it gives up and reports status 2 (the
// dense factor's flag waits sleep 64 ns per poll: ~0.5 s in all).
constexpr long long DEFAULT_WAIT_LIMIT = 1LL << 22;

struct DeviceProblem {
    int nc = 0, np = 0, no = 0, N = 0, Np = 0;  // N = cnp nc, Np = N padded to TILE
    int cnp = 6;                // parameters per camera: 6, 11 or 16
    int prec = PSBA_PREC_FP64;  // storage of the per-observation / per-point arrays (double or float)
    // problem (immutable)
    double *K = nullptr, *q0 = nullptr, *meas = nullptr;
    double *wt = nullptr;      // 3 per obs (a, b, c of L = [[a, b], [0, c]]), or null: unweighted
    int *obs_pt = nullptr, *obs_cam = nullptr;
    int *pt_start = nullptr;   // np + 1
    int *pt_order = nullptr;   // np: points by observation count, descending (per-point kernels' order)
    int2 *eb_warps = nullptr;  // eb/dpb warps: first slot in pt_order, m; padded to EB_WARPS, plus a sentinel
    int n_eb_warps = 0;
    int *cam_obs = nullptr;    // observations sorted by (camera, point)
    // camera pair lists for the off-diagonal Schur blocks (k > l)
    int n_pairs = 0;           // nonempty pairs
    int *pair_kl = nullptr;    // 2 per pair: k, l
    int *pair_a = nullptr;     // entries: observation of camera k
    int *pair_b = nullptr;     // entries: observation of camera l
    long long n_pair_entries = 0;
    // off-diagonal Schur work, two layouts whose partial slots are numbered in
    // pair-list order (each pair's slots form one range):
    // units of <= SCHUR_CHUNK entries of one pair, one slot each, longest
    // first (FP32 products, and 11/16-parameter cameras);
    SchurUnit *off_units = nullptr;
    int n_off_units = 0;
    int *off_unit_start = nullptr;  // per pair: first unit (n_pairs + 1)
    // 6-parameter cameras, FP64 products: the pair list cut into equal chunks
    // (SchurUnit: first pair, first entry, entries, first slot), one per thread
    // of one resident wave, a slot per pair a chunk touches
    SchurUnit *off_chunks = nullptr;
    int n_off_chunks = 0;
    // 6-parameter cameras, FP32 products: units of <= MX_UNIT entries of one
    // pair, one warp and one slot each, longest first
    SchurUnit *mx_units = nullptr;
    int n_mx_units = 0;
    int *mx_unit_start = nullptr;  // per pair: first unit (n_pairs + 1)
    int n_off_chunk_slots = 0;
    int *off_chunk_start = nullptr;  // per pair: first slot (n_pairs + 1)
    int *pair_start = nullptr;       // per pair: first entry (n_pairs + 1)
    SchurUnit *diag_units = nullptr;  // per camera chunks of cam_obs
    int n_diag_units = 0;
    int *diag_unit_start = nullptr;   // per camera (nc + 1)
    CamUnit *cam_units = nullptr;
    int n_cam_units = 0;
    int *cam_unit_start = nullptr;    // per camera (nc + 1)
    // parameters
    double *cams = nullptr, *pts = nullptr;
    double *cams0 = nullptr, *pts0 = nullptr;  // initial estimate as uploaded
    // per-linearization
    double *camtab = nullptr;     // nc CamTab
    double *camtab_new = nullptr; // nc CamTab at p + dp
    double *ex = nullptr;         // 2 per obs
    double *A = nullptr;          // 12 per obs
    double *B = nullptr;          // 6 per obs
    double *W = nullptr;          // 18 per obs
    double *U = nullptr;          // 36 per camera
    double *V = nullptr;          // 6 per point (00 01 02 11 12 22)
    double *g = nullptr;          // N + 3 np
    double *uvdiag = nullptr;     // N + 3 np
    double *cam_partial = nullptr;  // n_cam_units * 27
    // per-trial
    double *Vinv = nullptr;       // 6 per point
    float *Vinv2f = nullptr;      // 12 per point: V^-1 as FP32 pairs hi + lo (the mixed form's Y)
    float *gb32 = nullptr;        // 3 per point: gb rounded to FP32 (the mixed form's ea sums)
    float *camtab32 = nullptr;    // CAMTAB32 per camera: the table's M, D, fx, sk, fy in FP32 (mixed J)
    double *Y = nullptr;          // 18 per obs
    double *schur_partial = nullptr;  // off-diagonal slots (off_partial_slots), then the diagonal units'
    double *S = nullptr;          // Np x Np (lower)
    double *Ssave = nullptr;      // copy of S (trust-region modified-Cholesky fallback, refinement), Nm3 x Nm3
    // the fallback's matrix size: Np, or (N not a multiple of 3: 11/16-parameter
    // cameras) Np rounded up to a multiple of 3, the rows past Np identity
    int Nm3 = 0;
    double *rhs = nullptr;        // Np (ea on entry, y after the forward solve)
    double *xsol = nullptr;       // Np
    double *rsave = nullptr;      // Np: ea saved before the factor (refinement)
    float2 *dpa2f = nullptr;      // Np: dpa as FP32 pairs hi + lo (the mixed form's eb sums)
    float2 *meas2f = nullptr;     // 2 per obs: the measurements as FP32 pairs (the mixed trial cost)
    float2 *x2f = nullptr;        // 3 per point: the trial point pts + dpb as FP32 pairs (the mixed trial cost)
    float2 *tab2f = nullptr;      // RES_TAB2F per camera: the trial camera table's projection values as FP32 pairs
    double *Linv = nullptr;       // (Np / TILE) * TILE * TILE inverses of the diagonal blocks
    int *status = nullptr;        // Cholesky status word (0 ok, 1 not SPD, 2 wait budget exhausted)
    int *tickets = nullptr;       // 3 words, zero between launches: last-block tickets (eb/dpb, residual, |p|^2)
    int2 *chol_tasks = nullptr;   // helper tasks of the dense factor, in dependency order
    int chol_n_tasks = 0;
    int chol_grid_cap = 0;        // CTAs of the dense factor at most (0: one per SM)
    long long wait_limit = DEFAULT_WAIT_LIMIT;  // polls per device-side wait (dense factor flags, Y copies)
    double *chol_pre = nullptr;   // second-subdiagonal tiles before their solve (Np / TILE tiles)
    int *chol_flags = nullptr;    // one flag per dataflow task (value = epoch when done)
    int chol_n_flags = 0;
    double *dp = nullptr;         // N + 3 np
    double *eb = nullptr;         // 3 np
    double *red_partial = nullptr;  // reduction partials
    int red_partial_cap = 0;
    TrialScalars *scal = nullptr; // device scalars
    TrialScalars *scal_host = nullptr;  // pinned host mirror
    // trust region vectors
    double *vecPU = nullptr, *vecPB = nullptr, *vecP = nullptr, *jx1 = nullptr, *jx2 = nullptr;
    double *E = nullptr;
    double *tmp9 = nullptr;       // 9 per point (full 3x3 copies for the parity interface)
    size_t bytes = 0;
};

// Linearization: camera tables, residual, Jacobian, W, V, gb, U, ga.
// (with_d: the derivative tables D as well, which only the linearization reads)
void launch_cam_tables(const DeviceProblem &d, const double *cams, const double *dpa,
                       double *tab, cudaStream_t s, float *tab32 = nullptr, float2 *tab2f = nullptr,
                       int with_d = 0);
void launch_residual_df(const DeviceProblem &d, double *partial, int nblocks, double *sum_dst, cudaStream_t s);
void launch_split2f(const double *x, float2 *out, long long n, cudaStream_t s);
void launch_linearize(const DeviceProblem &d, double coeff, cudaStream_t s);
// the mixed form's linearization projects in double-float FP32 arithmetic
// (6-parameter cameras, unweighted): its camera table split by k_cam_tables
inline bool linearize_df(const DeviceProblem &d) { return d.prec == PSBA_PREC_MIXED && d.cnp == 6 && !d.wt; }
void launch_point_blocks(const DeviceProblem &d, double coeff, cudaStream_t s);
void launch_camera_blocks(const DeviceProblem &d, double coeff, cudaStream_t s);
// Residual only (ex, when ex_out is set) at the parameters given by tab,
// pts (+ dpb), and its sum of squares into *sum_dst (block partials in
// partial; the launch's last block sums them).
void launch_residual(const DeviceProblem &d, const double *tab, const double *pts,
                     const double *dpb, double *ex_out, double *partial, int nblocks,
                     double *sum_dst, cudaStream_t s);
int residual_blocks(const DeviceProblem &d);

// Damping trial: V^-1, Y, Schur complement, ea.
void launch_vinv(const DeviceProblem &d, double mu, cudaStream_t s);
void launch_yblocks(const DeviceProblem &d, cudaStream_t s);
// Per-device kernel attributes (dynamic shared-memory opt-ins); call with the
// device current before the first launch on it.
constexpr int MAX_DEVICES = 64;
int prepare_device_kernels();
void launch_schur(const DeviceProblem &d, double mu, cudaStream_t s);
void launch_schur_off(const DeviceProblem &d, cudaStream_t s);
// threads of one resident wave of the 6-parameter off-diagonal Schur kernel on this device
int schur_off_wave_threads();
// off-diagonal partial slots reserved ahead of the diagonal partials (the larger layout)
inline size_t off_partial_slots(const DeviceProblem &d)
{
    size_t n = (size_t)(d.n_off_units > d.n_off_chunk_slots ? d.n_off_units : d.n_off_chunk_slots);
    return n > (size_t)d.n_mx_units ? n : (size_t)d.n_mx_units;
}
void launch_schur_diag(const DeviceProblem &d, cudaStream_t s);
void launch_schur_reduce(const DeviceProblem &d, double mu, cudaStream_t s);
// Back-substitution: eb, dpb and partial sums for |dp|^2 and dp.(mu dp + g).
void launch_eb_dpb(const DeviceProblem &d, double mu, cudaStream_t s);
int eb_blocks(const DeviceProblem &d);
void launch_update_params(const DeviceProblem &d, cudaStream_t s);

// Deterministic reductions and vector helpers.
void launch_sum_partials(const double *partial, int n, double *dst, cudaStream_t s);
// |cams|^2 and |pts|^2 (into dst_cams, dst_pts) in one launch: nred blocks over the points, one over the
// cameras, the last block summing the points' partials in index order
void launch_param_norm(const DeviceProblem &d, int nred, double *partial, double *dst_cams, double *dst_pts,
                       cudaStream_t s);
void launch_finish_trial(const DeviceProblem &d, double mu, cudaStream_t s);
void launch_max_uvdiag(const DeviceProblem &d, double *dst, cudaStream_t s);
void launch_dot(const double *x, const double *y, long long n, double *partial, int nblocks,
                double *dst, cudaStream_t s);
void launch_jmultiply(const DeviceProblem &d, const double *x, double *out, cudaStream_t s);
void launch_axpby(double *out, const double *x, double a, const double *y, double b, long long n,
                  cudaStream_t s);
void launch_scale(double *out, const double *x, const double *num, const double *den,
                  double den_scale, double sign, long long n, cudaStream_t s);

// Dense reduced-camera solve (psba_dense.cu): factors S (Np x Np, lower) in
// place with the forward solve of rhs carried along (one cooperative
// launch), then the back solve into x_out; epoch must increase from launch
// to launch.
void launch_chol_dataflow(const DeviceProblem &d, int epoch, double *x_out, cudaStream_t s);
void launch_refine(const DeviceProblem &d, const double *Sc, int ld, const double *bc, double *x, cudaStream_t s);
// at most cap CTAs for a handle's dense factor (0: one per SM); for callers
// that run several handles side by side
void set_chol_grid_cap(psba_handle *h, int cap);
// the dense factor's helper tasks, in dependency order
void chol_task_list(int nb, std::vector<int2> &tasks);

// index lists on the GPU, psba_index.cu
void launch_pt_start(int np, int no, const int *obs_pt, int *pt_start, cudaStream_t s);
// cam_obs: CTA (k, s) writes camera k's observations of chunk s from
// off[k * n_chunks + s] on; cam_fill_chunk gives the chunk length
int cam_fill_chunk(int nc, int no);
void launch_cam_fill(int nc, int no, int chunk, const int *obs_cam, const int *off, int *cam_obs, cudaStream_t s);
// pair lists per segment of a camera's list (pair_segment_len observations):
// counts per (segment, l), then the entries from the host-scanned offsets
int pair_segment_len(int nc, int no);
void launch_pair_count(int nc, int nseg, int seg_len, const int *seg_cam, const int *seg_first, const int *cam_start,
                       const int *cam_obs, const int *obs_pt, const int *obs_cam, const int *pt_start, int *cnt,
                       cudaStream_t s);
void launch_pair_fill(int nc, int nseg, int seg_len, const int *seg_cam, const int *seg_first, const int *cam_start,
                      const int *cam_obs, const int *obs_pt, const int *obs_cam, const int *pt_start, const int *off,
                      int *pa, int *pb, cudaStream_t s);

// variable intrinsics (cnp 11 / 16), psba_varcam.cu
size_t varcam_cam_partial(int cnp);   // doubles per camera-unit partial
size_t varcam_diag_partial(int cnp);  // doubles per diagonal Schur-unit partial
void launch_linearize_v(const DeviceProblem &d, double coeff, cudaStream_t s);
void launch_camera_blocks_v(const DeviceProblem &d, double coeff, cudaStream_t s);
void launch_yblocks_v(const DeviceProblem &d, cudaStream_t s);
void launch_schur_off_v(const DeviceProblem &d, cudaStream_t s);
void launch_schur_diag_v(const DeviceProblem &d, cudaStream_t s);
void launch_schur_reduce_v(const DeviceProblem &d, double mu, cudaStream_t s);
void launch_eb_dpb_v(const DeviceProblem &d, double mu, int nblocks, cudaStream_t s);
void launch_jmultiply_v(const DeviceProblem &d, const double *x, double *out, cudaStream_t s);
void launch_residual_dist(const DeviceProblem &d, const double *tab, const double *pts, const double *dpb,
                          double *ex_out, double *partial, int nblocks, cudaStream_t s);
// Modified Cholesky (trust-region lambda fallback) and its diagonal correction.
constexpr int CM_MAX_CTAS = 256;  // CTAs of the modified Cholesky's cooperative launch, at most
size_t cholmod_work(int n);       // doubles of work it needs at size n
void launch_cholmod(double *S, int n, int ld, double *E, double *work, cudaStream_t s, int grid_cap = 0);

// Copies for the parity interface.
void launch_expand_V(const DeviceProblem &d, const double *V6, double *V9, cudaStream_t s);

}  // namespace psba

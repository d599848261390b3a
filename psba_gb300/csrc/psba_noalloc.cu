// Reprojection cost with no device allocation (psba_cost_noalloc).
//
// Some callers cannot allocate device memory at the moment they need a cost
// evaluation: code running while a CUDA stream is being captured into a graph
// (cudaMalloc is not allowed during capture), a serving loop that admits work
// against a fixed HBM budget and must not grow its footprint per request, or
// a host framework that owns all device memory and hands out only its own
// buffers.  This entry point evaluates the cost psba_eval_residual returns
// for an unweighted problem with 6-parameter cameras and fixed K (the
// reference's compute_exQT + compute_L2_sq) on arrays the caller already
// holds on the device, with its scratch in a fixed array that is part of the
// library image instead of a cudaMalloc'd buffer.  It takes no covariances
// and no 11/16-parameter cameras: for those, psba_eval_residual's cost
// differs from this one.
//
// The observation indices come from caller memory and are not seen by the
// host, so the kernel checks them: an observation whose point index is
// outside 0..n_pts-1 or whose camera index is outside 0..n_cams-1 is not
// read through, and it makes the result NaN.
//
// The scratch array is shared by every call on a device and keeps the last
// call's contents.  Calls that overlap on the GPU (two streams, or two host
// threads without ordering between them) race on it; callers must order
// their calls.  Every call overwrites all the scratch it reads (camera tables
// and one partial sum per block), so nothing has to start at zero.
#include <mutex>

#include "psba_internal.h"

namespace psba {
namespace noalloc {

// Limits of the fixed scratch: camera tables (CAMTAB doubles per camera) and one
// partial sum per 256 observations.
constexpr int MAX_CAMS = 1024;
constexpr long long MAX_OBS = 16LL * 1024 * 1024;
constexpr int THREADS = 256;
constexpr size_t TAB_DOUBLES = (size_t)MAX_CAMS * CAMTAB;
constexpr size_t PARTIAL_DOUBLES = (size_t)(MAX_OBS / THREADS);
constexpr size_t SCRATCH_DOUBLES = TAB_DOUBLES + PARTIAL_DOUBLES;  // under 1 MiB in total
static_assert(SCRATCH_DOUBLES * sizeof(double) <= (1u << 20), "scratch above 1 MiB");

// Every GPU that loads the library holds this array until the process exits.
static __device__ __align__(256) double g_scratch[SCRATCH_DOUBLES];

static double *g_ptr[MAX_DEVICES];
static std::mutex g_mu;

// Device address of g_scratch for the current device, looked up once per
// device with that device current.  Host code only ever passes this address
// to kernels; g_scratch itself is a host-side stand-in on the host.  The
// cached address assumes the device's primary context lives as long as the
// process (no cudaDeviceReset between calls).
static int scratch_address(double **out)
{
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return set_error(std::string("cudaGetDevice: ") + cudaGetErrorString(e)), PSBA_ERR_CUDA;
    if (dev < 0 || dev >= MAX_DEVICES) return set_error("device index out of range"), PSBA_ERR_ARG;
    std::lock_guard<std::mutex> lock(g_mu);
    if (!g_ptr[dev]) {
        double *p = nullptr;
        e = cudaGetSymbolAddress((void **)&p, g_scratch);
        if (e != cudaSuccess || !p)
            return set_error(std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e)), PSBA_ERR_CUDA;
        g_ptr[dev] = p;
    }
    *out = g_ptr[dev];
    return PSBA_OK;
}

// Camera rotation (q(v) (x) q0), translation and intrinsics into the table.
__global__ void k_tables(int nc, const double *__restrict__ K, const double *__restrict__ q0,
                         const double *__restrict__ cams, double *__restrict__ tab)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= nc) return;
    const double v0 = cams[6 * j], v1 = cams[6 * j + 1], v2 = cams[6 * j + 2];
    const double s0 = q0[4 * j], a1 = q0[4 * j + 1], a2 = q0[4 * j + 2], a3 = q0[4 * j + 3];
    const double sl = sqrt(1.0 - v0 * v0 - v1 * v1 - v2 * v2);
    const double s = sl * s0 - (a1 * v0 + a2 * v1 + a3 * v2);
    const double a = s0 * v0 + sl * a1 + a3 * v1 - a2 * v2;
    const double b = s0 * v1 + sl * a2 + a1 * v2 - a3 * v0;
    const double c = s0 * v2 + sl * a3 + a2 * v0 - a1 * v1;
    const double d = s * s - (a * a + b * b + c * c);
    double *o = tab + (size_t)CAMTAB * j;
    o[0] = d + 2 * a * a;       o[1] = 2 * (a * b - s * c); o[2] = 2 * (a * c + s * b);
    o[3] = 2 * (a * b + s * c); o[4] = d + 2 * b * b;       o[5] = 2 * (b * c - s * a);
    o[6] = 2 * (a * c - s * b); o[7] = 2 * (b * c + s * a); o[8] = d + 2 * c * c;
    o[36] = cams[6 * j + 3];
    o[37] = cams[6 * j + 4];
    o[38] = cams[6 * j + 5];
    const double *k = K + 5 * j;
    o[39] = k[0];
    o[40] = k[4];
    o[41] = k[1];
    o[42] = k[0] * k[3];
    o[43] = k[2];
}

// Squared residuals, one partial sum per block of THREADS observations.  An
// observation with an index out of range is skipped and contributes NaN.
__global__ void __launch_bounds__(THREADS) k_sq(int nc, int np, int no, const int *__restrict__ obs_pt,
                                                const int *__restrict__ obs_cam,
                                                const double *__restrict__ meas,
                                                const double *__restrict__ pts,
                                                const double *__restrict__ tab,
                                                double *__restrict__ partial)
{
    __shared__ double red[THREADS];
    const int o = blockIdx.x * blockDim.x + threadIdx.x;
    double sq = 0.0;
    if (o < no) {
        const int i = obs_pt[o], j = obs_cam[o];
        if (i < 0 || i >= np || j < 0 || j >= nc) {
            sq = NAN;
        } else {
            const double X0 = pts[3 * i], X1 = pts[3 * i + 1], X2 = pts[3 * i + 2];
            const double *T = tab + (size_t)CAMTAB * j;
            const double xc = T[0] * X0 + T[1] * X1 + T[2] * X2 + T[36];
            const double yc = T[3] * X0 + T[4] * X1 + T[5] * X2 + T[37];
            const double zc = T[6] * X0 + T[7] * X1 + T[8] * X2 + T[38];
            const double iz = 1.0 / zc;
            const double u = (T[39] * xc + T[40] * yc + T[41] * zc) * iz;
            const double v = (T[42] * yc + T[43] * zc) * iz;
            const double e0 = meas[2 * (size_t)o] - u, e1 = meas[2 * (size_t)o + 1] - v;
            sq = e0 * e0 + e1 * e1;
        }
    }
    red[threadIdx.x] = sq;
    __syncthreads();
    for (int st = THREADS / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) red[threadIdx.x] += red[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = red[0];
}

// Fixed-order sum of the block partials into *cost.
__global__ void k_total(const double *__restrict__ partial, int n, double *__restrict__ cost)
{
    __shared__ double r[THREADS];
    double a = 0.0;
    for (int k = threadIdx.x; k < n; k += THREADS) a += partial[k];
    r[threadIdx.x] = a;
    __syncthreads();
    for (int st = THREADS / 2; st > 0; st >>= 1) {
        if (threadIdx.x < st) r[threadIdx.x] += r[threadIdx.x + st];
        __syncthreads();
    }
    if (threadIdx.x == 0) *cost = r[0];
}

}  // namespace noalloc
}  // namespace psba

extern "C" int psba_cost_noalloc(int n_cams, int n_pts, int n_obs, const double *K, const double *q0, const double *cams,
                                 const double *pts, const double *meas, const int *obs_pt, const int *obs_cam,
                                 double *cost, void *stream)
{
    using namespace psba;
    using namespace psba::noalloc;
    if (n_cams <= 0 || n_cams > MAX_CAMS)
        return set_error("psba_cost_noalloc: n_cams must be in 1.." + std::to_string(MAX_CAMS)), PSBA_ERR_ARG;
    if (n_pts < 0) return set_error("psba_cost_noalloc: n_pts must be >= 0"), PSBA_ERR_ARG;
    if (n_obs < 0 || n_obs > MAX_OBS)
        return set_error("psba_cost_noalloc: n_obs must be in 0.." + std::to_string(MAX_OBS)), PSBA_ERR_ARG;
    if (!K || !q0 || !cams || !cost || (n_obs > 0 && (!pts || !meas || !obs_pt || !obs_cam)))
        return set_error("psba_cost_noalloc: null pointer"), PSBA_ERR_ARG;
    double *scratch = nullptr;
    const int r = scratch_address(&scratch);
    if (r != PSBA_OK) return r;
    cudaStream_t s = (cudaStream_t)stream;
    double *tab = scratch;
    double *partial = scratch + TAB_DOUBLES;
    const int nblocks = n_obs > 0 ? (n_obs + THREADS - 1) / THREADS : 1;
    k_tables<<<(n_cams + 127) / 128, 128, 0, s>>>(n_cams, K, q0, cams, tab);
    note_launch(1);
    k_sq<<<nblocks, THREADS, 0, s>>>(n_cams, n_pts, n_obs, obs_pt, obs_cam, meas, pts, tab, partial);
    note_launch(1);
    k_total<<<1, THREADS, 0, s>>>(partial, nblocks, cost);
    note_launch(1);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return set_error(std::string("psba_cost_noalloc launch: ") + cudaGetErrorString(e)), PSBA_ERR_CUDA;
    return PSBA_OK;
}

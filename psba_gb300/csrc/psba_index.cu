// Observation index lists built on the GPU: what the reference's
// generate_idxs (PSBA/misc.cpp:178-218) builds on the host as the dense
// blk_idx (P x C) and comm3DIdx (C x C x P) tables, here as compact lists:
//   pt_start   (P + 1)  each point's observation range (observations are
//                       sorted by point, then camera)
//   cam_obs    (O)      observation ids per camera, ascending point order,
//                       with cam_start (C + 1)
//   pair lists          for every camera pair k > l with common points, the
//                       (observation of k, observation of l) entries in
//                       ascending point order -- the order in which
//                       compute_S.cl:39-77 sums them
// Every list is produced in a fixed order (block-wide scans and in-chunk
// sorts keyed by position, no order-dependent atomics), so it is the same
// on every run and equal to the host construction entry for entry.
#include <algorithm>

#include "psba_internal.h"

namespace psba {

namespace {

constexpr int IX_THREADS = 256;

// Exclusive scan of one int per thread over the block (IX_THREADS threads);
// *total receives the sum.
__device__ int block_exscan(int v, int *total)
{
    __shared__ int warp_tot[IX_THREADS / 32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = lane < IX_THREADS / 32 ? warp_tot[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, d);
            if (lane >= d) t += y;
        }
        if (lane < IX_THREADS / 32) warp_tot[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    const int before = w > 0 ? warp_tot[w - 1] : 0;
    *total = warp_tot[IX_THREADS / 32 - 1];
    __syncthreads();
    return before + x - v;
}

// Ascending bitonic sort of IX_THREADS keys in shared memory (one per thread).
__device__ void block_sort(unsigned *keys)
{
    const int t = threadIdx.x;
    for (int size = 2; size <= IX_THREADS; size <<= 1)
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            __syncthreads();
            const int partner = t ^ stride;
            if (partner > t) {
                const bool up = (t & size) == 0;
                const unsigned a = keys[t], b = keys[partner];
                if ((a > b) == up) {
                    keys[t] = b;
                    keys[partner] = a;
                }
            }
        }
    __syncthreads();
}

__device__ int lower_bound_u(const unsigned *a, int n, unsigned v)
{
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

}  // namespace

// pt_start[i] = first observation of point i (lower bound in the sorted obs_pt)
__global__ void k_pt_start(int np, int no, const int *__restrict__ obs_pt, int *__restrict__ pt_start)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i > np) return;
    int lo = 0, hi = no;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (obs_pt[mid] < i) lo = mid + 1;
        else hi = mid;
    }
    pt_start[i] = lo;
}

// CTA (k, s): the observations of camera k in chunk s (observations
// [s * chunk, (s + 1) * chunk)), in ascending order, from off[k * n_chunks + s]
// on (a stable block-wide compaction; the host counts the chunks).
__global__ void __launch_bounds__(IX_THREADS) k_cam_fill(int no, int chunk, const int *__restrict__ obs_cam,
                                                          const int *__restrict__ off, int *__restrict__ cam_obs)
{
    const int k = blockIdx.x, s = blockIdx.y;
    const int o0 = s * chunk, o1 = min(no, o0 + chunk);
    int base = off[(size_t)k * gridDim.y + s];
    for (int c0 = o0; c0 < o1; c0 += IX_THREADS) {
        const int o = c0 + threadIdx.x;
        const int f = (o < o1 && obs_cam[o] == k) ? 1 : 0;
        int total;
        const int pos = block_exscan(f, &total);
        if (f) cam_obs[base + pos] = o;
        base += total;
    }
}

// Pair entries are produced per segment: up to seg_len consecutive
// observations of one camera's list (camera seg_cam[q], from seg_first[q] in
// cam_obs).  For each observation a of camera k (point i), the earlier
// observations b of point i belong to cameras l < k: the entries (a, b) of
// pair (k, l).

// CTA per segment: its entries per pair (k, l), row q of cnt (nc wide).
__global__ void __launch_bounds__(IX_THREADS) k_pair_count(int nc, int seg_len, const int *__restrict__ seg_cam,
                                                            const int *__restrict__ seg_first,
                                                            const int *__restrict__ cam_start,
                                                            const int *__restrict__ cam_obs,
                                                            const int *__restrict__ obs_pt,
                                                            const int *__restrict__ obs_cam,
                                                            const int *__restrict__ pt_start, int *__restrict__ cnt)
{
    extern __shared__ int hist[];  // nc
    const int q = blockIdx.x, k = seg_cam[q];
    for (int l = threadIdx.x; l < nc; l += IX_THREADS) hist[l] = 0;
    __syncthreads();
    const int first = seg_first[q], end = min(cam_start[k + 1], first + seg_len);
    for (int idx = first + threadIdx.x; idx < end; idx += IX_THREADS) {
        const int a = cam_obs[idx];
        for (int b = pt_start[obs_pt[a]]; b < a; ++b) atomicAdd(&hist[obs_cam[b]], 1);  // integer counts
    }
    __syncthreads();
    for (int l = threadIdx.x; l < nc; l += IX_THREADS) cnt[(size_t)q * nc + l] = hist[l];
}

// CTA per segment: write its entries of every pair (k, l) from off[q * nc + l]
// on, in ascending point order.  The segment is taken IX_THREADS observations
// at a time; their entry stream (the observations in order, each followed by
// the earlier observations of its point) is cut into chunks of IX_THREADS
// entries, a chunk is sorted by (l, position), and each entry goes to its
// pair's running offset plus its rank among the chunk's entries of that pair.
__global__ void __launch_bounds__(IX_THREADS) k_pair_fill(int nc, int seg_len, const int *__restrict__ seg_cam,
                                                           const int *__restrict__ seg_first,
                                                           const int *__restrict__ cam_start,
                                                           const int *__restrict__ cam_obs,
                                                           const int *__restrict__ obs_pt,
                                                           const int *__restrict__ obs_cam,
                                                           const int *__restrict__ pt_start,
                                                           const int *__restrict__ off, int *__restrict__ pa,
                                                           int *__restrict__ pb)
{
    extern __shared__ int run[];  // nc running offsets
    __shared__ int goff[IX_THREADS], ga[IX_THREADS], eA[IX_THREADS], eB[IX_THREADS];
    __shared__ unsigned keys[IX_THREADS];
    const int q = blockIdx.x, k = seg_cam[q], t = threadIdx.x;
    for (int l = t; l < nc; l += IX_THREADS) run[l] = off[(size_t)q * nc + l];
    const int first = seg_first[q], end = min(cam_start[k + 1], first + seg_len);
    for (int o0 = first; o0 < end; o0 += IX_THREADS) {
        const int idx = o0 + t;
        int g = 0, a = -1;
        if (idx < end) {
            a = cam_obs[idx];
            g = a - pt_start[obs_pt[a]];
        }
        int total;
        const int ex = block_exscan(g, &total);  // its barriers also order run[] and the previous pass
        goff[t] = ex;
        ga[t] = a;
        __syncthreads();
        for (int e0 = 0; e0 < total; e0 += IX_THREADS) {
            const int e = e0 + t;
            unsigned key = 0xffffffffu;
            if (e < total) {
                // owner: the last observation whose entries start at or before e
                int lo = 0, hi = IX_THREADS;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (goff[mid] <= e) lo = mid + 1;
                    else hi = mid;
                }
                const int j = lo - 1;
                const int aa = ga[j];
                const int b = pt_start[obs_pt[aa]] + (e - goff[j]);
                eA[t] = aa;
                eB[t] = b;
                key = ((unsigned)obs_cam[b] << 8) | (unsigned)t;
            }
            keys[t] = key;
            block_sort(keys);
            const unsigned v = keys[t];
            int l = -1, lo_l = 0;
            if (v != 0xffffffffu) {
                l = (int)(v >> 8);
                lo_l = lower_bound_u(keys, IX_THREADS, (unsigned)l << 8);
                const int src = (int)(v & 0xffu);
                const int dest = run[l] + (t - lo_l);
                pa[dest] = eA[src];
                pb[dest] = eB[src];
            }
            __syncthreads();
            if (l >= 0 && (t == IX_THREADS - 1 || (keys[t + 1] >> 8) != (unsigned)l)) run[l] += t - lo_l + 1;
            __syncthreads();
        }
    }
}

void launch_pt_start(int np, int no, const int *obs_pt, int *pt_start, cudaStream_t s)
{
    k_pt_start<<<(np + 1 + 255) / 256, 256, 0, s>>>(np, no, obs_pt, pt_start);
    note_launch(1);
}

int cam_fill_chunk(int nc, int no)
{
    // 8 passes of IX_THREADS per CTA, more when nc x chunks would pass 4M or
    // the chunks the grid's 65535 rows
    const long long want = std::max(((long long)no * nc + (1LL << 22) - 1) >> 22, ((long long)no + 65534) / 65535);
    const long long c = std::max<long long>(8 * IX_THREADS, (want + IX_THREADS - 1) / IX_THREADS * IX_THREADS);
    return (int)std::min<long long>(c, std::max(no, IX_THREADS));
}

void launch_cam_fill(int nc, int no, int chunk, const int *obs_cam, const int *off, int *cam_obs, cudaStream_t s)
{
    if (no == 0) return;
    k_cam_fill<<<dim3(nc, (no + chunk - 1) / chunk), IX_THREADS, 0, s>>>(no, chunk, obs_cam, off, cam_obs);
    note_launch(1);
}

int pair_segment_len(int nc, int no)
{
    // one pass of IX_THREADS per CTA, more when segments x nc would pass 4M
    const long long m = std::max<long long>(1, ((long long)no * nc + (256LL << 22) - 1) / (256LL << 22));
    return (int)std::min<long long>(m * IX_THREADS, 1 << 30);
}

void launch_pair_count(int nc, int nseg, int seg_len, const int *seg_cam, const int *seg_first, const int *cam_start,
                       const int *cam_obs, const int *obs_pt, const int *obs_cam, const int *pt_start, int *cnt,
                       cudaStream_t s)
{
    if (nseg == 0) return;
    k_pair_count<<<nseg, IX_THREADS, sizeof(int) * nc, s>>>(nc, seg_len, seg_cam, seg_first, cam_start, cam_obs,
                                                            obs_pt, obs_cam, pt_start, cnt);
    note_launch(1);
}

void launch_pair_fill(int nc, int nseg, int seg_len, const int *seg_cam, const int *seg_first, const int *cam_start,
                      const int *cam_obs, const int *obs_pt, const int *obs_cam, const int *pt_start, const int *off,
                      int *pa, int *pb, cudaStream_t s)
{
    if (nseg == 0) return;
    k_pair_fill<<<nseg, IX_THREADS, sizeof(int) * nc, s>>>(nc, seg_len, seg_cam, seg_first, cam_start, cam_obs, obs_pt,
                                                           obs_cam, pt_start, off, pa, pb);
    note_launch(1);
}

}  // namespace psba

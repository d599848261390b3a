// Shared between the batched solver (psba_batch.cu) and the serving engine
// (psba_serve.cu): the per-problem table entry, the resumable LM state, and
// the host helpers that lay a problem out in the arenas.
#pragma once

#include <string>
#include <vector>

#include "psba_internal.h"

namespace psba {
namespace batch {

struct BatchProblem {
    int nc, np, no, N;
    int n_pairs, flags;  // flags: low byte = lanes per camera pair in the Schur stage (0 = 32)
    int slice, pad_;     // outer LM iterations per launch (0: run to the end)
    long long d_K, d_q0, d_cams, d_pts, d_cams0, d_pts0, d_meas;                 // double arena
    long long i_obs_pt, i_obs_cam, i_pt_start, i_cam_start, i_cam_obs, i_pair_start, i_pair_kl, i_pair_a,
        i_pair_b;                                                                  // int arena
    long long r_ex, r_A, r_B, r_W, r_Y;                                            // R arena
    // R arena, used by the mixed form only (as FP32 values and FP32 pairs): the
    // Jacobian's FP32 camera table, the projection's split tables (current,
    // trial), the split measurements, current and trial points, V^-1, the
    // camera step, and gb rounded to FP32
    long long r_tab32, r_tab2f, r_tab2f2, r_meas2f, r_pts2f, r_x2f, r_vinv2f, r_dpa2f, r_gb32;
    long long d_V, d_Vinv, d_U, d_g, d_uvdiag, d_dp, d_S, d_tab, d_tab2, d_rhs, d_x;  // double arena
};

// A problem's LM state between launches (and its result at the end): the
// driver's scalars, saved at an outer-iteration boundary.  Parameters stay in
// the arena; the linearisation is rebuilt from them at the start of each
// outer iteration, so resuming gives the same bits as running straight on.
struct BatchResult {
    int status, iterations, trials, linearizations;
    double initial_cost, final_cost, mu;  // final_cost: the current cost while running
    double p_L2;
    int nu, first, started, pad;
};

struct BatchOpts {
    double tau, stop_thresh, eps;
    int max_iter, allow_switch, precision, pad;
};

// Host layout of one problem with offsets counted from zero in each arena:
// nd doubles (initialised content in dA, the rest zero), ni ints (iA) and nr
// elements of the per-observation type.  Returns false with a message when
// the description is malformed.
struct ProblemLayout {
    BatchProblem bp;
    std::vector<double> dA;
    std::vector<int> iA;
    long long nr = 0;
    double work = 0.0;  // relative cost of one LM iteration (scheduling weight)
};
bool build_problem_layout(const psba_problem_desc &desc, ProblemLayout &out, std::string &err);

// Move a problem's offsets by (dbase, ibase, rbase) elements.
void rebase_problem(BatchProblem &bp, long long dbase, long long ibase, long long rbase);

// Bytes of one problem in a single byte pool: doubles, then ints, then the
// per-observation arrays, each part starting 256-byte aligned.
size_t pool_bytes(const ProblemLayout &L, int precision);

// The persistent launch over problems probs[order[0..n)] with state in res[];
// all three arenas point into one byte pool when called from the server.
cudaError_t launch_batch_lm(int precision, int grid, int threads, cudaStream_t s, const BatchProblem *probs,
                            const int *order, int n, int *queue, double *darena, int *iarena, void *rarena,
                            const BatchOpts *opts, BatchResult *res);
int batch_blocks_per_sm(int precision, int threads);

}  // namespace batch
}  // namespace psba

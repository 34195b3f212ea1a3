// Parameters of the persistent SIRT kernel (sirt.cu): a table of independent
// problems, each a stack of slices that share one geometry.
#pragma once

#include "synk_internal.cuh"
#include "fp_tile.cuh"

namespace synk {

struct SirtProblem {
    ProbGeom P;
    AngleLists L;         // angle order of the lane-per-angle projector
    const float *R;       // [a*D] row normaliser (shared by the slices); negative = a listed corner ray
    const int2 *graze;    // [4*graze_capc] rays that only clip a corner pixel, {k, r}, corner c at c*graze_capc
    const float *glen;    // [4*graze_capc] their chords (the reference's f32 sums)
    float *gcontrib;      // [nslices][4*graze_capc] their backprojection terms chord*R*e
    const int *goff;      // device [5]: corner c's entries are goff[c+1] - goff[c], prefix order
    const float *C;       // [N*N] column normaliser
    const float *b;       // [nslices][a*D] sinograms
    float *xpad;          // [nslices][N][N+2] iterate, zero column on each side
    float *xTpad;         // [nslices][N][N+2] transposed iterate, same padding
    float *rr;            // [nslices][a*D] weighted residual R*(b - FP(x))
    float *rrp;           // [nslices][a*D] its detector pairs (rr[s], rr[s+1]) per row (0 past the row end)
                          // for the backprojection-grid backward phase; null when that phase does not run
    double *res2;         // [nslices][iterations+1] sum of (b - FP(x_k))^2
    const double *b2;     // [nslices] ||b||^2
    int *stop_iter;       // [nslices] iteration at which the stopping rule fired (init: INT_MAX)
    double *residuals;    // optional out [nslices][iterations+1]: sqrt(res2/b2)
    int *iters_done;      // optional out [nslices]
    int nslices;
    int iterations;
    int fp_split;         // 1,2,4,8 warps share one ray (rows split)
    int bp_split;         // 1,2,4,8 warps share one pixel (angles split)
    int bp_pix;           // 1,2,4 pixels (rows) per thread in the backward phase
    int bp_inrange;       // every pixel's detector window is inside the sinogram (no bounds checks)
    int graze_capc;       // capacity of one corner's list
    // filled on the device by sirt_plan_kernel (they depend on the angle lists)
    int fp_ips;           // FP work items per slice
    int bp_ips;           // BP work items per slice
    long long fp_begin;   // first global FP item of this problem
    long long bp_begin;   // first global BP item of this problem
};

struct SirtParams {
    SirtProblem *probs;   // [nprob] (device)
    long long *totals;    // [2] FP and BP items of all problems (device, from sirt_plan_kernel)
    int nprob;
    int max_iterations;
    unsigned *bar;        // [2] barrier arrival count and generation
    unsigned *work;       // [3] rotating work counters (dynamic assignment)
    int *status;          // SYNK_OK or SYNK_ETIMEOUT
    unsigned long long timeout_ns;
    unsigned barrier_extra;   // blocks the grid barrier waits for beyond the grid (fault injection; 0)
    double tol2;          // relative tolerance squared (0: no stopping rule)
    int record_final;     // also measure the residual of each problem's final iterate
    int dynamic;          // hand out items with an atomic counter (uneven batches)
};

cudaError_t launch_sumsq(const float *b, size_t len, int nslices, double *out, cudaStream_t stream);
cudaError_t launch_sirt_plan(SirtProblem *probs, int nprob, long long *totals, cudaStream_t stream);
int sirt_persistent_grid(int *blocks_per_sm);
cudaError_t launch_sirt_persistent(const SirtParams &p, int grid, cudaStream_t stream);
// phase-split engine: resident grids of the two phase kernels, and their launches
int sirt_phase_grids(int *fp_grid, int *bp_grid);
cudaError_t launch_sirt_fp_phase(const SirtParams &p, int it, int grid, cudaStream_t stream);
cudaError_t launch_sirt_bp_phase(const SirtParams &p, int it, int *active, int grid, cudaStream_t stream);
// forward phase of the split engine for one problem (a slice stack): the projector's grid, residual epilogue
cudaError_t launch_sirt_fp_stack(const SirtProblem &q, int it, double tol2, int record_final, cudaStream_t stream);
// backward phase of the split engine for one problem on the backprojector's tile grid (needs q.rrp and every
// detector window of its 64-row tiles inside the sinogram); block (0,0,0) applies the stopping rule into *active
cudaError_t launch_sirt_bp_stack(const SirtProblem &q, int it, double tol2, int *active, cudaStream_t stream);
cudaError_t launch_sirt_finalize(SirtProblem *probs, int nprob, int max_slices, int record_final,
                                 cudaStream_t stream);

}  // namespace synk

// Parameters of the persistent SIRT kernel (sirt.cu).
#pragma once

#include "synk_internal.cuh"
#include "fp_tile.cuh"

namespace synk {

struct SirtParams {
    ProbGeom P;
    const float *R;       // [a*D] row normaliser (shared by all slices)
    const float *C;       // [N*N] column normaliser
    AngleLists L;         // angle order of the lane-per-angle projector
    const float *b;       // [nslices][a*D] sinograms
    float *xpad;          // [nslices][N][N+2] iterate, zero column on each side
    float *xTpad;         // [nslices][N][N+2] transposed iterate, same padding
    float *rr;            // [nslices][a*D] weighted residual R*(b - FP(x))
    double *res2;         // [nslices][iterations+1] sum of (b - FP(x_k))^2
    const double *b2;     // [nslices] ||b||^2
    int *stop_iter;       // [nslices] iteration at which the stopping rule fired (init: iterations)
    unsigned *bar;        // [2] barrier arrival count and generation
    int *status;          // SYNK_OK or SYNK_ETIMEOUT
    unsigned long long timeout_ns;
    double tol2;          // relative tolerance squared (0: no stopping rule)
    int nslices;
    int iterations;
    int record_final;     // also measure the residual of the final iterate
    int fp_split;         // 1,2,4,8 warps share one ray (rows split)
    int bp_split;         // 1,2,4,8 warps share one pixel (angles split)
};

cudaError_t launch_sumsq(const float *b, size_t len, int nslices, double *out, cudaStream_t stream);
int sirt_persistent_grid(int *blocks_per_sm);
cudaError_t launch_sirt_persistent(const SirtParams &p, int grid, cudaStream_t stream);
cudaError_t launch_sirt_finalize(const SirtParams &p, double *residuals, int *iters_done, cudaStream_t stream);

}  // namespace synk

// CSR system-matrix kernels (csr.cu).
#pragma once

#include "synk_internal.cuh"

namespace synk {

// counts[rows] of A (transpose=false: rows are rays) or A^T (rows are pixels)
cudaError_t launch_csr_count(const ProbGeom &P, bool transpose, int *counts, cudaStream_t st);
// offsets[rows+1] = exclusive scan of counts, offsets[rows] = total
cudaError_t exclusive_scan(const int *counts, int64_t n, int64_t *offsets, int64_t *scratch_sums,
                           int64_t *total, cudaStream_t st);
cudaError_t launch_csr_fill(const ProbGeom &P, bool transpose, const int64_t *ptr, int *idx, float *vals,
                            cudaStream_t st);
// y = M x for an n-row CSR matrix with int64 (ptr64) or int32 (ptr32) row pointers
cudaError_t launch_spmv(int64_t rows, const int64_t *ptr64, const int *ptr32, const int *idx, const float *vals,
                        const float *x, float *y, cudaStream_t st);

}  // namespace synk

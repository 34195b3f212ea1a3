// CSR system-matrix path (no counterpart in the reference): the forward
// projector's rule (futhark/forwardprojection.fut:31-56) stored as a sparse
// matrix A (rays x pixels) and its transpose A^T (pixels x rays), and the two
// sparse matrix-vector products y = A*x, x = A^T*y.
//
// Both matrices are built on the GPU from the same per-(ray, frame row)
// rule that the on-the-fly projector evaluates:
//   A   ray by ray:     count -> exclusive scan -> fill (entries in traversal order)
//   A^T pixel by pixel: for every angle, the few rays whose traversal of the
//                       pixel's frame row reaches the pixel are found from the
//                       ray geometry and the rule is re-evaluated for them, so
//                       every value is bit-identical to A's and each row of A^T
//                       lists its rays in ascending order (deterministic sums).
// SpMV: one warp per row, four independent 128-byte loads in flight per warp
// (HBM-bound: 8 bytes per non-zero plus the row pointers and the gathered
// vector, which stays in L2).
#include <math.h>

#include "synk_internal.cuh"
#include "csr_internal.cuh"

namespace synk {

// Entries of ray r of angle g in frame row j (0-based): up to two
// (frame column, weight) pairs, weight 0 meaning "no entry".
struct RowEntries {
    int c0, c1;
    float w0, w1;
};

__device__ __forceinline__ float ray_intercept(const ProbGeom &P, const AngleGeom &g, int r, float *rho_out) {
    const float rho = __fadd_rn(P.rhozero, __fmul_rn((float)r, P.deltarho));
    if (rho_out) *rho_out = rho;
    return __fdiv_rn(rho, g.cost);
}

// The forward rule at one frame row, fast path (see fp_rows_fast).
__device__ __forceinline__ RowEntries row_fast(const ProbGeom &P, const AngleGeom &g, float u0, int j) {
    RowEntries e;
    const float u = fmaf((float)j, g.slope, u0);
    int c;
    const float fl = floor_magic(u, c);
    const float t = right_share(u, fl, g.ainv);
    e.c0 = c;
    e.c1 = c + 1;
    e.w0 = ((unsigned)c < (unsigned)P.N) ? __fmul_rn(__fsub_rn(1.0f, t), g.lbase) : 0.0f;
    e.w1 = ((unsigned)(c + 1) < (unsigned)P.N) ? __fmul_rn(t, g.lbase) : 0.0f;
    return e;
}

// The forward rule at one frame row, the reference's own expressions.
__device__ __forceinline__ RowEntries row_exact(const ProbGeom &P, const AngleGeom &g, float intercept, int j) {
    RowEntries e;
    const int half = P.half;
    const int i = j - half;
    const float xbot = __fadd_rn(__fmul_rn((float)i, g.slope), intercept);
    const float xtop = __fadd_rn(xbot, g.slope);
    const int xpb = (int)floorf(xbot);
    const int xpt = (int)floorf(xtop);
    const float xpmax = (float)max(xpb, xpt);
    const float xdiff = __fsub_rn(xtop, xbot);
    const bool single = xpb == xpt;
    const bool botin = xpb >= -half && xpb < half;
    const bool topin = (!single) && xpt >= -half && xpt < half;
    const float lxbot = single ? g.lbase : __fmul_rn(__fdiv_rn(__fsub_rn(xpmax, xbot), xdiff), g.lbase);
    const float lxtop = __fmul_rn(__fdiv_rn(__fsub_rn(xtop, xpmax), xdiff), g.lbase);
    e.c0 = xpb + half;
    e.c1 = xpt + half;
    e.w0 = botin ? lxbot : 0.0f;
    e.w1 = topin ? lxtop : 0.0f;
    return e;
}

__device__ __forceinline__ bool ray_in_range(const ProbGeom &P, float rho) {
    return !(fabsf(rho) > 0.75f * (float)P.N + 2.0f);
}

// Frame row range of a fast-path ray (as fp_ray clips it).
__device__ __forceinline__ void fast_rows(const ProbGeom &P, const AngleGeom &g, float u0, int &j0, int &j1) {
    j0 = 0;
    j1 = P.N;
    const float aslope = fabsf(g.slope);
    if (g.slope != 0.0f) {
        const float ja = (-1.0f - aslope - u0) / g.slope;
        const float jb = ((float)P.N - u0) / g.slope;
        float lo = fmaxf(fminf(ja, jb) - 1.0f, 0.0f);
        float hi = fminf(fmaxf(ja, jb) + 2.0f, (float)P.N);
        j0 = (int)lo;
        j1 = (hi > lo) ? (int)hi : j0;
    } else if (!(u0 > -1.0f && u0 < (float)P.N)) {
        j1 = j0;
    }
}

__device__ __forceinline__ int64_t pixel_of(const ProbGeom &P, const AngleGeom &g, int j, int c) {
    return g.flat ? (int64_t)c * P.N + j : (int64_t)j * P.N + c;
}

// ---- A: ray-driven count and fill ----------------------------------------------
template <bool FILL>
__global__ void __launch_bounds__(256) ray_entries_kernel(ProbGeom P, int *__restrict__ counts,
                                                          const int64_t *__restrict__ rowptr,
                                                          int *__restrict__ colidx, float *__restrict__ vals) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = blockIdx.y * 8 + warp;
    const int r = blockIdx.x * 32 + lane;
    if (k >= P.a || r >= P.D) return;
    const AngleGeom g = load_geom(P.geom, k);
    const int64_t ray = (int64_t)k * P.D + r;
    float rho;
    const float intercept = ray_intercept(P, g, r, &rho);
    int64_t pos = FILL ? rowptr[ray] : 0;
    int cnt = 0;
    if (ray_in_range(P, rho)) {
        int j0 = 0, j1 = P.N;
        float u0 = 0.0f;
        if (!g.exact) {
            u0 = ray_u0(P, g, intercept);
            fast_rows(P, g, u0, j0, j1);
        }
        for (int j = j0; j < j1; ++j) {
            const RowEntries e = g.exact ? row_exact(P, g, intercept, j) : row_fast(P, g, u0, j);
            if (e.w0 != 0.0f) {
                if (FILL) { colidx[pos] = (int)pixel_of(P, g, j, e.c0); vals[pos] = e.w0; ++pos; }
                ++cnt;
            }
            if (e.w1 != 0.0f) {
                if (FILL) { colidx[pos] = (int)pixel_of(P, g, j, e.c1); vals[pos] = e.w1; ++pos; }
                ++cnt;
            }
        }
    }
    if (!FILL) counts[ray] = cnt;
}

// ---- A^T: pixel-driven count and fill --------------------------------------------
// For pixel (row, col) and angle k, the frame row is j and the frame column c.
// A ray's traversal reaches column c at row j when its left end u (fast path)
// lies in [c-1, c+1), or when one of its two pixels xpb/xpt is c (exact path):
// u is monotonic in the detector index with step deltarho/cost, so a short
// window of detectors around the solution of u = c holds every candidate.
template <bool FILL>
__global__ void __launch_bounds__(256) pixel_entries_kernel(ProbGeom P, int *__restrict__ counts,
                                                            const int64_t *__restrict__ colptr,
                                                            int *__restrict__ rowidx, float *__restrict__ vals) {
    const int col = blockIdx.x * 32 + (threadIdx.x & 31);
    const int row = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (row >= P.N || col >= P.N) return;
    const int64_t pix = (int64_t)row * P.N + col;
    int64_t pos = FILL ? colptr[pix] : 0;
    int cnt = 0;
    for (int k = 0; k < P.a; ++k) {
        const AngleGeom g = load_geom(P.geom, k);
        const int j = g.flat ? col : row;
        const int c = g.flat ? row : col;
        // u(r) = j*slope + (rhozero + r*deltarho)/cost + slope_lo + half - half*slope
        // exact path, frame column of xbot: (j-half)*slope + (rhozero + r*deltarho)/cost + half
        const double du = (double)P.deltarho / (double)g.cost;            // du/dr
        const double base = g.exact ? (double)(j - P.half) * g.slope + (double)P.rhozero / g.cost + P.half
                                    : (double)j * g.slope + (double)P.rhozero / g.cost + g.slope_lo + P.half -
                                          (double)P.half * g.slope;
        // window in u (frame-column coordinates): [c - 2, c + 2]
        double ra = ((double)c - 2.0 - base) / du, rb = ((double)c + 2.0 - base) / du;
        if (ra > rb) { const double t = ra; ra = rb; rb = t; }
        int r0 = (int)floor(ra) - 1, r1 = (int)ceil(rb) + 1;
        r0 = max(r0, 0);
        r1 = min(r1, P.D - 1);
        for (int r = r0; r <= r1; ++r) {
            float rho;
            const float intercept = ray_intercept(P, g, r, &rho);
            if (!ray_in_range(P, rho)) continue;
            RowEntries e;
            if (g.exact) {
                e = row_exact(P, g, intercept, j);
            } else {
                const float u0 = ray_u0(P, g, intercept);
                int j0, j1;
                fast_rows(P, g, u0, j0, j1);
                if (j < j0 || j >= j1) continue;
                e = row_fast(P, g, u0, j);
            }
            const int64_t ray = (int64_t)k * P.D + r;
            if (e.w0 != 0.0f && e.c0 == c) {
                if (FILL) { rowidx[pos] = (int)ray; vals[pos] = e.w0; ++pos; }
                ++cnt;
            }
            if (e.w1 != 0.0f && e.c1 == c) {
                if (FILL) { rowidx[pos] = (int)ray; vals[pos] = e.w1; ++pos; }
                ++cnt;
            }
        }
    }
    if (!FILL) counts[pix] = cnt;
}

// ---- exclusive scan of int counts into int64 offsets (three passes) -----------
constexpr int kScanBlock = 1024;

__global__ void scan_blocks_kernel(const int *__restrict__ in, int64_t n, int64_t *__restrict__ out,
                                   int64_t *__restrict__ block_sums) {
    __shared__ int64_t sh[kScanBlock];
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    const int64_t v = i < n ? in[i] : 0;
    sh[threadIdx.x] = v;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
        const int64_t t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
        __syncthreads();
        sh[threadIdx.x] += t;
        __syncthreads();
    }
    if (i < n) out[i] = sh[threadIdx.x] - v;    // exclusive
    if (threadIdx.x == kScanBlock - 1) block_sums[blockIdx.x] = sh[threadIdx.x];
}

__global__ void scan_sums_kernel(int64_t *__restrict__ sums, int64_t nb, int64_t *__restrict__ total) {
    // one block, sequential over chunks of kScanBlock
    __shared__ int64_t sh[kScanBlock];
    int64_t carry = 0;
    for (int64_t b0 = 0; b0 < nb; b0 += kScanBlock) {
        const int64_t i = b0 + threadIdx.x;
        const int64_t v = i < nb ? sums[i] : 0;
        sh[threadIdx.x] = v;
        __syncthreads();
        for (int off = 1; off < kScanBlock; off <<= 1) {
            const int64_t t = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
            __syncthreads();
            sh[threadIdx.x] += t;
            __syncthreads();
        }
        if (i < nb) sums[i] = carry + sh[threadIdx.x] - v;
        const int64_t chunk = sh[kScanBlock - 1];
        __syncthreads();
        carry += chunk;
    }
    if (threadIdx.x == 0) *total = carry;
}

__global__ void scan_add_kernel(int64_t *__restrict__ out, int64_t n, const int64_t *__restrict__ sums,
                                const int64_t *__restrict__ total) {
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    if (i < n) out[i] += sums[blockIdx.x];
    if (i == n - 1) out[n] = *total;
}

cudaError_t exclusive_scan(const int *counts, int64_t n, int64_t *offsets, int64_t *scratch_sums,
                           int64_t *total, cudaStream_t st) {
    const int64_t nb = (n + kScanBlock - 1) / kScanBlock;
    scan_blocks_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(counts, n, offsets, scratch_sums);
    scan_sums_kernel<<<1, kScanBlock, 0, st>>>(scratch_sums, nb, total);
    scan_add_kernel<<<(unsigned)nb, kScanBlock, 0, st>>>(offsets, n, scratch_sums, total);
    return cudaGetLastError();
}

cudaError_t launch_csr_count(const ProbGeom &P, bool transpose, int *counts, cudaStream_t st) {
    if (!transpose) {
        dim3 grid((P.D + 31) / 32, (P.a + 7) / 8);
        ray_entries_kernel<false><<<grid, 256, 0, st>>>(P, counts, nullptr, nullptr, nullptr);
    } else {
        dim3 grid((P.N + 31) / 32, (P.N + 7) / 8);
        pixel_entries_kernel<false><<<grid, 256, 0, st>>>(P, counts, nullptr, nullptr, nullptr);
    }
    return cudaGetLastError();
}

cudaError_t launch_csr_fill(const ProbGeom &P, bool transpose, const int64_t *ptr, int *idx, float *vals,
                            cudaStream_t st) {
    if (!transpose) {
        dim3 grid((P.D + 31) / 32, (P.a + 7) / 8);
        ray_entries_kernel<true><<<grid, 256, 0, st>>>(P, nullptr, ptr, idx, vals);
    } else {
        dim3 grid((P.N + 31) / 32, (P.N + 7) / 8);
        pixel_entries_kernel<true><<<grid, 256, 0, st>>>(P, nullptr, ptr, idx, vals);
    }
    return cudaGetLastError();
}

// ---- SpMV ----------------------------------------------------------------------
// y[row] = sum_k vals[k] * x[idx[k]] over rowptr[row] <= k < rowptr[row+1];
// one warp per row, rows handed out grid-stride.  The streams of indices and
// values run one 128-entry chunk (and one row's pointers) ahead of the x
// gathers, so a warp keeps HBM reads in flight while it waits on a gather.
// The entries past a row's end hold value 0 and index 0, and their gathers
// run unpredicated: predicating them cost 5-25 % of the bandwidth on GB300.
// 0 * x[0] adds nothing while x[0] is finite; when it is not, the kernel
// takes the predicated walk, so a non-finite x[0] reaches only the rows that
// hold column 0.  With the launch below, A*x at N=512, 512 angles streams
// 5.0 TB/s (4.3 before the look-ahead), A^T*y 5.0 (3.8).
template <bool GUARD, class PtrT>
__device__ __forceinline__ void spmv_rows(int64_t rows, const PtrT *__restrict__ ptr, const int *__restrict__ idx,
                                          const float *__restrict__ vals, const float *__restrict__ x,
                                          float *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
    int64_t row = (int64_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (row >= rows) return;
    int64_t b = (int64_t)ptr[row], e = (int64_t)ptr[row + 1];
    for (; row < rows; row += warps) {
        // the next row's pointers, fetched while this row streams
        const int64_t nrow = row + warps;
        int64_t nb = 0, ne = 0;
        if (nrow < rows) {
            nb = (int64_t)ptr[nrow];
            ne = (int64_t)ptr[nrow + 1];
        }
        float acc0 = 0.0f, acc1 = 0.0f, acc2 = 0.0f, acc3 = 0.0f;
        int64_t k = b + lane;
        // chunk of 128 entries: lane l holds entries k, k+32, k+64, k+96
        int i0 = 0, i1 = 0, i2 = 0, i3 = 0;
        float v0 = 0.0f, v1 = 0.0f, v2 = 0.0f, v3 = 0.0f;
        if (k < e) { i0 = __ldcs(idx + k); v0 = __ldcs(vals + k); }
        if (k + 32 < e) { i1 = __ldcs(idx + k + 32); v1 = __ldcs(vals + k + 32); }
        if (k + 64 < e) { i2 = __ldcs(idx + k + 64); v2 = __ldcs(vals + k + 64); }
        if (k + 96 < e) { i3 = __ldcs(idx + k + 96); v3 = __ldcs(vals + k + 96); }
        for (; k < e; k += 128) {
            const int64_t kn = k + 128;
            int j0 = 0, j1 = 0, j2 = 0, j3 = 0;
            float w0 = 0.0f, w1 = 0.0f, w2 = 0.0f, w3 = 0.0f;
            if (kn < e) { j0 = __ldcs(idx + kn); w0 = __ldcs(vals + kn); }
            if (kn + 32 < e) { j1 = __ldcs(idx + kn + 32); w1 = __ldcs(vals + kn + 32); }
            if (kn + 64 < e) { j2 = __ldcs(idx + kn + 64); w2 = __ldcs(vals + kn + 64); }
            if (kn + 96 < e) { j3 = __ldcs(idx + kn + 96); w3 = __ldcs(vals + kn + 96); }
            acc0 = fmaf(v0, __ldg(x + i0), acc0);
            if (!GUARD || k + 32 < e) acc1 = fmaf(v1, __ldg(x + i1), acc1);
            if (!GUARD || k + 64 < e) acc2 = fmaf(v2, __ldg(x + i2), acc2);
            if (!GUARD || k + 96 < e) acc3 = fmaf(v3, __ldg(x + i3), acc3);
            i0 = j0; i1 = j1; i2 = j2; i3 = j3;
            v0 = w0; v1 = w1; v2 = w2; v3 = w3;
        }
        float acc = (acc0 + acc1) + (acc2 + acc3);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (lane == 0) y[row] = acc;
        b = nb;
        e = ne;
    }
}

template <class PtrT>
__global__ void __launch_bounds__(256) spmv_warp_kernel(int64_t rows, const PtrT *__restrict__ ptr,
                                                        const int *__restrict__ idx, const float *__restrict__ vals,
                                                        const float *__restrict__ x, float *__restrict__ y) {
    // x[0] exists whenever a row holds an entry (its index is a column of x)
    if (rows > 0 && ptr[rows] > ptr[0] && !isfinite(__ldg(x)))
        spmv_rows<true>(rows, ptr, idx, vals, x, y);
    else
        spmv_rows<false>(rows, ptr, idx, vals, x, y);
}

cudaError_t launch_spmv(int64_t rows, const int64_t *ptr64, const int *ptr32, const int *idx, const float *vals,
                        const float *x, float *y, cudaStream_t st) {
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    // 64 blocks of 8 warps per SM, about 5 waves of resident blocks: the
    // hardware hands blocks to the SMs that finish first, which evens out the
    // rows' unequal lengths.  Measured at N=512, 512 angles (A*x / A^T*y, ms):
    // 8 per SM 0.331/0.339, 16 0.308/0.314, 32 0.279/0.287, 64 0.273/0.277,
    // 128 0.277/0.273, one block per 8 rows 0.304/0.279.
    const int64_t want = (rows + 7) / 8, cap = (int64_t)sms * 64;
    const int grid = (int)(want < cap ? (want > 0 ? want : 1) : cap);
    if (ptr64) spmv_warp_kernel<int64_t><<<grid, 256, 0, st>>>(rows, ptr64, idx, vals, x, y);
    else spmv_warp_kernel<int><<<grid, 256, 0, st>>>(rows, ptr32, idx, vals, x, y);
    return cudaGetLastError();
}

}  // namespace synk

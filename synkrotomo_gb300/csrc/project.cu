// Projector kernels of libsynk: per-angle geometry table, image transpose,
// ray-driven forward projector, pixel-driven backprojector and the SIRT
// normalisers R = 1/(A*1), C = 1/(A^T*1).
//
// Forward projector (futhark/forwardprojection.fut:21-84): one thread per ray,
// one warp per 32 consecutive detectors of one angle, eight angles per block
// so that the eight warps of a block gather from overlapping image rows.  Flat
// lines walk the transposed image, as the reference does, which keeps every
// warp's gathers on one image row.
//
// Backprojector (futhark/backprojection.fut:19-93): one thread per pixel, a
// 32 x 8 pixel tile per block, all angles in a loop; the pixel's chord with
// each candidate ray is evaluated from the ray's distance to the pixel centre
// (a trapezoid in rho), which is the reference's intersect_fact*lbase
// (backprojection.fut:22-33, 62) without its per-detector divisions.
// Near-axis lines keep the reference's own expressions (see geometry_kernel).
#include <math.h>

#include "synk_internal.cuh"

namespace synk {

// sirtlib.fut:28-44 per angle, plus the constants of both traversals.  cos
// and sin are evaluated in FP64 and rounded once, so they are the correctly
// rounded float32 values that the reference's f32.cos / f32.sin return for
// all practical inputs.
__global__ void geometry_kernel(const float *__restrict__ angles, int a, AngleGeom *__restrict__ geom) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a) return;
    const double th = (double)angles[k];
    const float c = (float)cos(th);
    const float s = (float)sin(th);
    const bool flat = fabsf(s) >= fabsf(c);                       // sirtlib.fut:6-7
    const float q1 = __fdiv_rn(s, c), q2 = __fdiv_rn(c, s);
    const float lsteep = __fsqrt_rn(__fadd_rn(1.0f, __fmul_rn(q1, q1)));   // sirtlib.fut:33
    const float lflat = __fsqrt_rn(__fadd_rn(1.0f, __fmul_rn(q2, q2)));    // sirtlib.fut:34
    AngleGeom g;
    g.cost = flat ? -s : c;                                       // sirtlib.fut:41
    g.sint = flat ? c : -s;
    g.lbase = flat ? lflat : lsteep;
    g.slope = __fdiv_rn(-g.sint, g.cost);                         // forwardprojection.fut:26
    g.c = c;
    g.s = s;
    const float ac = fabsf(c), as = fabsf(s);
    const float amax = fmaxf(ac, as), bmin = fminf(ac, as);
    const float h = 0.5f * (amax + bmin);
    g.inv_b = bmin > 1.0f / kCap ? 1.0f / bmin : kCap;
    g.h_over_b = h * g.inv_b;
    g.slope_lo = fminf(g.slope, 0.0f);
    const float asl = fabsf(g.slope);
    g.ainv = asl > 1.0f / kCap ? 1.0f / asl : kCap;
    g.flat = flat ? 1 : 0;
    // Near-axis lines: with |slope| this small a ray can stay on a pixel edge
    // over the whole image (integer rho at theta = 0 or pi/2), and which
    // column receives it depends on how the reference's f32 expressions
    // round.  Those few angles run the reference's expressions verbatim.
    g.exact = asl < kExactSlope ? 1 : 0;
    geom[k] = g;
}

cudaError_t launch_geometry(const float *angles, int a, AngleGeom *geom, cudaStream_t stream) {
    geometry_kernel<<<(a + 127) / 128, 128, 0, stream>>>(angles, a, geom);
    return cudaGetLastError();
}

// out[z][c][r] = in[z][r][c], N x N slices.
__global__ void transpose_kernel(const float *__restrict__ in, float *__restrict__ out, int N) {
    __shared__ float tile[32][33];
    const size_t off = (size_t)blockIdx.z * N * N;
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int r = by + y, c = bx + threadIdx.x;
        if (r < N && c < N) tile[y][threadIdx.x] = in[off + (size_t)r * N + c];
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int c = bx + y, r = by + threadIdx.x;
        if (r < N && c < N) out[off + (size_t)c * N + r] = tile[threadIdx.x][y];
    }
}

cudaError_t launch_transpose(const float *in, float *out, int N, int nslices, cudaStream_t stream) {
    dim3 grid((N + 31) / 32, (N + 31) / 32, nslices);
    transpose_kernel<<<grid, dim3(32, 8), 0, stream>>>(in, out, N);
    return cudaGetLastError();
}

// Forward projection: ONES=false writes the ray sums, ONES=true writes the
// normaliser R = safe_inverse(A*1) (SIRT.fut:22-23, sirtlib.fut:9-13).
template <bool ONES>
__global__ void __launch_bounds__(256) fp_kernel(ProbGeom P, const float *__restrict__ img,
                                                 const float *__restrict__ imgT, float *__restrict__ out) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = blockIdx.y * 8 + warp;
    const int r = blockIdx.x * 32 + lane;
    if (k >= P.a || r >= P.D) return;
    const AngleGeom g = load_geom(P.geom, k);
    const float *frame = g.flat ? imgT : img;
    const auto v = fp_ray<ONES>(P, g, frame, r, 0, P.N);
    if constexpr (ONES) out[(size_t)k * P.D + r] = v != 0.0 ? (float)(1.0 / v) : 0.0f;
    else out[(size_t)k * P.D + r] = v;
}

cudaError_t launch_fp(const ProbGeom &P, const float *img, const float *imgT, float *sino, cudaStream_t stream) {
    dim3 grid((P.D + 31) / 32, (P.a + 7) / 8);
    fp_kernel<false><<<grid, 256, 0, stream>>>(P, img, imgT, sino);
    return cudaGetLastError();
}

// Backprojection: ONES=false writes the image, ONES=true writes the normaliser
// C = safe_inverse(A^T*1) (SIRT.fut:25) with the angle sum in FP64.
template <bool ONES>
__global__ void __launch_bounds__(256) bp_kernel(ProbGeom P, const float *__restrict__ sino, float *__restrict__ out) {
    const int col = blockIdx.x * 32 + (threadIdx.x & 31);
    const int row = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (row >= P.N || col >= P.N) return;
    float sum = 0.0f, comp = 0.0f;
    double dsum = 0.0;
    for (int k0 = 0; k0 < P.a; k0 += 32) {
        const int k1 = min(k0 + 32, P.a);
        float part = 0.0f;
        for (int k = k0; k < k1; ++k) {
            const AngleGeom g = load_geom(P.geom, k);
            part += bp_angle<ONES>(P, g, sino + (size_t)k * P.D, row, col);
        }
        if constexpr (ONES) dsum += (double)part;
        else comp_add(sum, comp, part);
    }
    if constexpr (ONES) out[(size_t)row * P.N + col] = dsum != 0.0 ? (float)(1.0 / dsum) : 0.0f;
    else out[(size_t)row * P.N + col] = sum + comp;
}

cudaError_t launch_bp(const ProbGeom &P, const float *sino, float *img, cudaStream_t stream) {
    dim3 grid((P.N + 31) / 32, (P.N + 7) / 8);
    bp_kernel<false><<<grid, 256, 0, stream>>>(P, sino, img);
    return cudaGetLastError();
}

cudaError_t launch_normalisers(const ProbGeom &P, float *R, float *C, cudaStream_t stream) {
    dim3 gf((P.D + 31) / 32, (P.a + 7) / 8);
    fp_kernel<true><<<gf, 256, 0, stream>>>(P, nullptr, nullptr, R);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dim3 gb((P.N + 31) / 32, (P.N + 7) / 8);
    bp_kernel<true><<<gb, 256, 0, stream>>>(P, nullptr, C);
    return cudaGetLastError();
}

}  // namespace synk

// Ray-driven forward projection with one lane per angle, shared by the
// standalone forward projector and the SIRT kernels.
//
// A lane owns one ray (detector r, angle k); the lanes of a warp hold
// neighbouring rays of the same class (all steep or all flat, none
// near-axis): 32 angles at one detector, or 4 angles x 8 detectors in the
// standalone projector.  Neighbouring rays cross almost the same pixels of a
// frame row, so each gather of a row touches few sectors (32 adjacent
// detectors of one angle would span ~45 columns; 4 x 8 averages fewest).  The
// walk takes the warp's union of the lanes' row ranges.  Two image layouts:
//   fp_lane_ray_pair (standalone projector): pair images, entry i of a row =
//     (pixel i-1, pixel i - pixel i-1) with zeros outside the image and a zero
//     entry ending the row; one unconditional 8-byte gather per row step.
//   fp_lane_ray (SIRT, whose iterate is kept padded): row stride N+2, a zero
//     column on each side, so one predicate covers both 4-byte gathers.
// Per lane and row (forwardprojection.fut:31-56):
//   x  = (j - half)*slope + x0         left end of the row segment, centred
//   c  = floor(x) + half, t = max(0, (x - floor(x) + |slope| - 1) / |slope|)   share of c+1
//   s += v[c] + t*(v[c+1] - v[c])      (times lbase once per ray)
// Near-axis angles are listed separately and run the reference's own
// expressions (fp_exact in project.cu / the SIRT kernel).
#pragma once

#include "synk_internal.cuh"

namespace synk {

// Rows per partial sum of a ray before it enters the compensated (Neumaier)
// total: plain float32 within a chunk, compensated across chunks.  Longer
// chunks mean fewer compensation steps and a tighter row loop; measured at
// N=2048 / 2048 angles, the standalone projector takes 4.54 / 4.34 / 4.22 /
// 4.17 ms with 32 / 64 / 128 / 256 rows, and the SIRT slice stack (N=512,
// 360 angles) 107.8 / 106.7 / 105.8 us per slice-iteration with 32 / 64 /
// 128 (the last with 128-angle backprojection chunks).  A float32 partial
// sum of n terms errs by at most (n - 1) * 2^-24 of the terms' absolute sum,
// so 256 rows stay far inside the 1e-5 parity bar, and a 2048-row ray still
// gets 8 compensated chunks.
constexpr int kPairCompRows = 256;
constexpr int kSirtCompRows = 128;

// Angle order of the lane-per-angle projector (built by angle_lists_kernel):
//   order[g*32 + lane]: angle of lane in group g, -1 for an idle lane;
//   groups [0, counts[0]) are steep, [counts[0], counts[0]+counts[1]) flat;
//   exact[0 .. counts[2]): the near-axis angles.
struct AngleLists {
    const int *order;
    const int *exact;
    const int *counts;   // device: steep groups, flat groups, near-axis angles
};

// Row range [j0, j1) in which the ray's segment can touch a column of [0, N)
// (x0: ray_x0).
__device__ __forceinline__ void lane_rows(const ProbGeom &P, const AngleGeom &g, float x0, int &j0, int &j1) {
    ray_rows(P, g, x0, j0, j1);
}

// Ray sum of detector r for angle geometry g by one thread with the
// reference's own expressions (forwardprojection.fut:31-56), rows in the
// reference's order and float32 accumulation, so the value is the f32
// reference's bit for bit.  img_frame points at pixel (0, 0) of the frame
// image (the transposed image for flat lines), rows `stride` floats apart;
// ONES reads no image.  Rows whose segment cannot touch the image add exactly
// zero in the reference and are skipped (the fast path's row clip with its
// margins).  Used for the chords of rays that clip one corner pixel, which the
// two float32 formulations round differently enough to matter once SIRT
// divides by them.
template <bool ONES>
__device__ __forceinline__ float fp_ray_exact_f32(const ProbGeom &P, const AngleGeom &g,
                                                  const float *__restrict__ img_frame, int stride, int r) {
    const float rho = __fadd_rn(P.rhozero, __fmul_rn((float)r, P.deltarho));    // forwardprojection.fut:28
    if (fabsf(rho) > 0.75f * (float)P.N + 2.0f) return 0.0f;
    const float intercept = __fdiv_rn(rho, g.cost);                               // forwardprojection.fut:29
    int j0 = 0, j1 = P.N;
    if (!g.exact) lane_rows(P, g, ray_x0(g, intercept), j0, j1);
    float acc = 0.0f;
    for (int j = j0; j < j1; ++j)
        acc = __fadd_rn(acc, fp_row_exact<ONES>(img_frame, stride, P.half, g.slope, intercept, g.lbase, j - P.half));
    return acc;
}

// fp_lane_ray: the sum over frame rows [jb, je) of detector r for the lane's
// angle k (k < 0: idle lane, returns 0) on the padded frame image, in two
// parts.  lane_ray_prep reads only the problem's static tables (geometry,
// detector positions), so a kernel can run it before waiting for the kernel
// that writes the image; the walk's row range is the warp's union of the
// lanes' ranges.  All 32 lanes of the warp must call both.
struct LaneRay {
    float x0, slope, ainv, lbase;
    int J0, J1;
    bool valid;
};

__device__ __forceinline__ LaneRay lane_ray_prep(const ProbGeom &P, int k, int r, int jb, int je) {
    const AngleGeom g = load_geom(P.geom, k >= 0 ? k : 0);
    const float rho = __fadd_rn(P.rhozero, __fmul_rn((float)r, P.deltarho));    // forwardprojection.fut:28
    const float intercept = __fdiv_rn(rho, g.cost);                               // forwardprojection.fut:29
    LaneRay L;
    L.x0 = ray_x0(g, intercept);
    int j0 = 0, j1 = 0;
    if (k >= 0 && !(fabsf(rho) > 0.75f * (float)P.N + 2.0f)) lane_rows(P, g, L.x0, j0, j1);
    j0 = max(j0, jb);
    j1 = min(j1, je);
    if (j1 <= j0) { j0 = je; j1 = je; }
    L.J0 = __reduce_min_sync(0xffffffffu, j0);
    L.J1 = __reduce_max_sync(0xffffffffu, j1);
    L.slope = g.slope;
    L.ainv = g.ainv;
    L.lbase = g.lbase;
    L.valid = k >= 0;
    return L;
}

// The walk of a prepared ray over the padded frame image img_pad (stride N+2,
// pixel (j, c) at j*(N+2) + c + 1); returns 0 for an idle lane.
__device__ __forceinline__ float fp_lane_walk(const ProbGeom &P, const LaneRay &L, const float *__restrict__ img_pad) {
    const float x0 = L.x0, slope = L.slope, ainv = L.ainv;
    const int J0 = L.J0, J1 = L.J1;
    const int stride = P.N + 2;
    const unsigned lim = (unsigned)P.N;     // c + 1 in [0, N]
    const int half = P.half;
    // floor(x) + half straight from the bits: x + (kMagic + half) rounded down
    // holds it in the low mantissa bits (kMagic + half is an exact float)
    const float magic_h = kMagic + (float)half;
    // x of rows j..j+3 from one float row counter: x0 + k*slope per lane
    const float x1 = x0 + slope, x2 = x0 + 2.0f * slope, x3 = x0 + 3.0f * slope;
    float sum = 0.0f, comp = 0.0f;
    auto row = [&](float x, int jrow, float &part) {
        const float rr = __fadd_rd(x, magic_h);
        const int c = __float_as_int(rr) - kMagicBits;     // pixel index floor(x) + half
        const float fl = __fsub_rn(rr, magic_h);             // floor(x)
        const float t = right_share(x, fl, ainv);
        const bool ok = (unsigned)(c + 1) <= lim;
        const float *p = img_pad + (jrow * stride + c + 1);
        const float v0 = ok ? __ldg(p) : 0.0f;
        const float v1 = ok ? __ldg(p + 1) : 0.0f;
        part += fmaf(t, v1 - v0, v0);
    };
    for (int j = J0; j < J1;) {
        const int jend = min(j + kSirtCompRows, J1);
        float part = 0.0f;
        float jf = (float)(j - half);
        for (; j + 3 < jend; j += 4, jf += 4.0f) {
            row(fmaf(jf, slope, x0), j, part);
            row(fmaf(jf, slope, x1), j + 1, part);
            row(fmaf(jf, slope, x2), j + 2, part);
            row(fmaf(jf, slope, x3), j + 3, part);
        }
        for (; j < jend; ++j, jf += 1.0f) row(fmaf(jf, slope, x0), j, part);
        comp_add(sum, comp, part);
    }
    return L.valid ? (sum + comp) * L.lbase : 0.0f;
}

__device__ __forceinline__ float fp_lane_ray(const ProbGeom &P, int k, int r, const float *__restrict__ img_pad,
                                             int jb, int je) {
    const LaneRay L = lane_ray_prep(P, k, r, jb, je);
    return fp_lane_walk(P, L, img_pad);
}

// fp_lane_ray on a pair image: pair[j*(N+2) + i] = (pad(j, i), pad(j, i+1) -
// pad(j, i)) for i in [0, N+1], where pad(j, i) = pixel (j, i-1) and 0 outside
// [1, N]; entry N+1 of every row is (0, 0).  One 8-byte gather per row serves
// both pixels of the row segment (v0 + t*(v1 - v0) is one FMA on the entry).
// Its index comes from the bits of r = x + kMagic rounded down,
// c + 1 = bits(r) - (kMagicBits - 1 - half), clamped as unsigned to N+1: a segment
// left of column -1 wraps to a huge value and one right of N-1 exceeds N, and
// both read the zero entry.  The loads are unconditional, so the rows of one
// unrolled step issue their gathers back to back.
__device__ __forceinline__ float fp_lane_ray_pair(const ProbGeom &P, int k, int r, const float2 *__restrict__ pair,
                                                  int jb, int je) {
    const AngleGeom g = load_geom(P.geom, k >= 0 ? k : 0);
    const float rho = __fadd_rn(P.rhozero, __fmul_rn((float)r, P.deltarho));    // forwardprojection.fut:28
    const float intercept = __fdiv_rn(rho, g.cost);                               // forwardprojection.fut:29
    const float x0 = ray_x0(g, intercept);
    int j0 = 0, j1 = 0;
    if (k >= 0 && !(fabsf(rho) > 0.75f * (float)P.N + 2.0f)) lane_rows(P, g, x0, j0, j1);
    j0 = max(j0, jb);
    j1 = min(j1, je);
    if (j1 <= j0) { j0 = je; j1 = je; }
    const int J0 = __reduce_min_sync(0xffffffffu, j0);
    const int J1 = __reduce_max_sync(0xffffffffu, j1);
    const float slope = g.slope, ainv = g.ainv;
    const uintptr_t rowbytes = (uintptr_t)(P.N + 2) * 8u;
    const unsigned zix = (unsigned)P.N + 1u;                   // the zero entry of a row
    // bits(r) - okbase = c + 1 with c = floor(x) + half the pixel index
    const unsigned okbase = (unsigned)kMagicBits - 1u - (unsigned)P.half;
    const uintptr_t base = reinterpret_cast<uintptr_t>(pair);
    const float x1 = x0 + slope, x2 = x0 + 2.0f * slope, x3 = x0 + 3.0f * slope;
    float sum = 0.0f, comp = 0.0f;
    auto row = [&](float x, uintptr_t rowb, float &part) {
        const float rr = __fadd_rd(x, kMagic);
        const float fl = __fsub_rn(rr, kMagic);
        const float t = right_share(x, fl, ainv);
        const unsigned ix = min((unsigned)__float_as_int(rr) - okbase, zix);
        const float2 v = __ldg(reinterpret_cast<const float2 *>(rowb + (uintptr_t)ix * 8u));
        part += fmaf(t, v.y, v.x);
    };
    for (int j = J0; j < J1;) {
        const int jend = min(j + kPairCompRows, J1);
        float part = 0.0f;
        float jf = (float)(j - P.half);
        uintptr_t rowb = base + (uintptr_t)j * rowbytes;
        for (; j + 3 < jend; j += 4, jf += 4.0f, rowb += 4 * rowbytes) {
            row(fmaf(jf, slope, x0), rowb, part);
            row(fmaf(jf, slope, x1), rowb + rowbytes, part);
            row(fmaf(jf, slope, x2), rowb + 2 * rowbytes, part);
            row(fmaf(jf, slope, x3), rowb + 3 * rowbytes, part);
        }
        for (; j < jend; ++j, jf += 1.0f, rowb += rowbytes) row(fmaf(jf, slope, x0), rowb, part);
        comp_add(sum, comp, part);
    }
    return k >= 0 ? (sum + comp) * g.lbase : 0.0f;
}

// Ray of a near-axis angle k, the reference's own expressions
// (forwardprojection.fut:31-56), computed by the 32 lanes of a warp over the
// frame rows [jb, je): lane l takes rows jb+l, jb+l+32, ...; the lane sums are
// combined in a fixed order.  Returns the sum in every lane.
// ESTEP 1: plain padded images (row stride N+2); ESTEP 2: pair images read
// through their first halves (row stride 2*(N+2) floats).
template <int ESTEP = 1>
__device__ __forceinline__ float fp_exact_ray_warp(const ProbGeom &P, int k, int r, const float *__restrict__ xpad,
                                                   const float *__restrict__ xTpad, int jb = 0, int je = 1 << 30) {
    const int lane = threadIdx.x & 31;
    const AngleGeom g = load_geom(P.geom, k);
    const float rho = __fadd_rn(P.rhozero, __fmul_rn((float)r, P.deltarho));
    if (fabsf(rho) > 0.75f * (float)P.N + 2.0f) return 0.0f;
    const float intercept = __fdiv_rn(rho, g.cost);
    const float *img = (g.flat ? xTpad : xpad) + ESTEP;
    const int stride = ESTEP == 1 ? P.N + 2 : 2 * (P.N + 2);
    float acc = 0.0f;
    const int iend = min(P.half, -P.half + je);
    for (int i = -P.half + jb + lane; i < iend; i += 32)
        acc = __fadd_rn(acc, fp_row_exact<false, ESTEP>(img, stride, P.half, g.slope, intercept, g.lbase, i));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
    return acc;
}

cudaError_t launch_angle_lists(const ProbGeom &P, int *order, int *exact, int *counts, cudaStream_t stream);
cudaError_t launch_pad(const float *x, float *xpad, float *xTpad, int N, int nslices, cudaStream_t stream);
// geometry table + angle lists (+ the pair images of x when x is not null) in one launch
cudaError_t launch_setup(const float *angles, int a, AngleGeom *geom, int *order, int *exact, int *counts,
                         const float *x, float2 *xpair, float2 *xTpair, int N, cudaStream_t stream);
cudaError_t launch_unpad(const float *xpad, float *x, int N, int nslices, cudaStream_t stream);

}  // namespace synk

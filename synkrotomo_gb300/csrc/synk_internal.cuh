// Internal device-side definitions shared by the projector, SIRT and CSR
// kernels of libsynk.  Geometry convention (futhark/forwardprojection.fut:26-29,
// futhark/sirtlib.fut:41): the ray of angle theta and detector r is the line
// rho = x*cos(theta) - y*sin(theta), rho = rhozero + r*deltarho, with
// x = col - N/2, y = row - N/2 and pixel (row, col) = [x, x+1) x [y, y+1).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/synk.h"

namespace synk {

// ---------------------------------------------------------------------------
// Per-angle geometry table (48 bytes, read as three float4 by the kernels).
// ---------------------------------------------------------------------------
struct __align__(16) AngleGeom {
    // Reference line triple in the traversal frame (sirtlib.fut:41): steep
    // lines (cos, -sin, lsteep) on the image, flat lines (-sin, cos, lflat)
    // on the transposed image.
    float cost, sint, lbase, slope;   // slope = -sint/cost (forwardprojection.fut:26)
    // Chord-length trapezoid in the true frame: for a pixel whose centre has
    // rho_c, a ray at rho has length lbase * sat((h - |rho - rho_c|) / b) with
    // a = max(|cos|,|sin|), b = min(|cos|,|sin|), h = (a+b)/2.
    float c, s, h_over_b, inv_b;      // cos, sin, h/b, 1/b (both capped)
    // Forward traversal constants and path selection.
    float slope_lo;    // min(slope, 0): xlo = xbot + slope_lo
    float ainv;        // 1/|slope| (capped)
    int   flat;        // 1: the line traverses the transposed image
    int   exact;       // 1: near-axis line, evaluate the reference's own formulas
};
static_assert(sizeof(AngleGeom) == 48, "AngleGeom layout");

// |slope| below this uses the reference's own f32 expression order (see
// geometry.cu): there a ray can run along a pixel edge for its whole length
// and the rounding of the reference's expressions decides which column gets it.
constexpr float kExactSlope = 1.0f / 4096.0f;
constexpr float kCap = 1.0e30f;

// sqrt(2)/2 evaluated as the reference does in f32 (backprojection.fut:20).
__host__ __device__ inline float fact_f32() { return 0.70710677f; }

// ---------------------------------------------------------------------------
// Floor without the conversion unit (Blackwell's F2I/FRND issue at a quarter
// of the FP32 rate).  Adding 1.5*2^23 with round-toward-minus-infinity leaves
// floor(x) in the low mantissa bits for |x| < 2^22 (the classic "magic number"
// rounding of IEEE-754 single precision): two FP32 adds and an integer add.
// ---------------------------------------------------------------------------
constexpr float kMagic = 12582912.0f;     // 1.5 * 2^23
constexpr int kMagicBits = 0x4B400000;

__device__ __forceinline__ float floor_magic(float x, int &ix) {
    const float r = __fadd_rd(x, kMagic);
    ix = __float_as_int(r) - kMagicBits;
    return __fsub_rn(r, kMagic);
}
__device__ __forceinline__ float ceil_magic(float x, int &ix) {
    const float r = __fadd_ru(x, kMagic);
    ix = __float_as_int(r) - kMagicBits;
    return __fsub_rn(r, kMagic);
}

// Neumaier-compensated accumulation of a block partial into (sum, comp).
__device__ __forceinline__ void comp_add(float &sum, float &comp, float v) {
    const float t = __fadd_rn(sum, v);
    if (fabsf(sum) >= fabsf(v)) comp = __fadd_rn(comp, __fadd_rn(__fsub_rn(sum, t), v));
    else comp = __fadd_rn(comp, __fadd_rn(__fsub_rn(v, t), sum));
    sum = t;
}

// ---------------------------------------------------------------------------
// One 2D problem as the kernels see it.
// ---------------------------------------------------------------------------
struct ProbGeom {
    int N;          // image is N x N (N even)
    int half;       // N/2
    int a;          // angles
    int D;          // detectors per angle (numrhos)
    int rpp;        // rhos per pixel: ceil(sqrt(2)/deltarho) (backprojection.fut:87)
    float rhozero;
    float deltarho;
    float inv_deltarho;
    // Centred detector coordinate: detector s = s' + zi sits at rz_c + s'*deltarho,
    // rz_c = rhozero + zi*deltarho, |rz_c| <= deltarho/2.  The backprojector
    // measures rho from rz_c rather than rhozero, so its coordinate stays below
    // ~N/sqrt(2) in magnitude (half the rounding of one running up to D).
    int zi;
    float rz_c;
    const AngleGeom *geom;   // [a]
};

// Left end of a fast-path ray's segment in frame row 0, in pixel-index units:
// u0 = intercept + min(slope,0) + half - half*slope (the CSR builders' walk,
// whose matrix and transpose are built from this one expression).
__device__ __forceinline__ float ray_u0(const ProbGeom &P, const AngleGeom &g, float intercept) {
    const float halff = (float)P.half;
    return __fmaf_rn(-halff, g.slope, __fadd_rn(__fadd_rn(intercept, g.slope_lo), halff));
}

// Left end of a fast-path ray's segment in the centred frame, at the middle
// row (i = j - half = 0): x0 = intercept + min(slope, 0); row j's segment
// starts at x = (j - half)*slope + x0 and column floor(x) + half.  The
// projectors and SIRT walk rays with it: |x| stays within ~N/2 on the rows a
// ray crosses, so it rounds half as coarsely as the pixel-index coordinate.
__device__ __forceinline__ float ray_x0(const AngleGeom &g, float intercept) {
    return __fadd_rn(intercept, g.slope_lo);
}

// Frame rows [j0, j1) whose segment [x, x + |slope|] can touch a column of
// the image, for a ray starting at x0 (ray_x0); one row of margin below and
// two above absorb the rounding.
__device__ __forceinline__ void ray_rows(const ProbGeom &P, const AngleGeom &g, float x0, int &j0, int &j1) {
    j0 = 0;
    j1 = P.N;
    const float halff = (float)P.half;
    const float aslope = fabsf(g.slope);
    if (g.slope != 0.0f) {
        const float ja = halff + (-1.0f - aslope - halff - x0) / g.slope;
        const float jb = halff + (halff - x0) / g.slope;
        const float lo = fmaxf(fminf(ja, jb) - 1.0f, 0.0f);
        const float hi = fminf(fmaxf(ja, jb) + 2.0f, (float)P.N);
        j0 = (int)lo;
        j1 = (hi > lo) ? (int)hi : j0;
    } else if (!(x0 > -1.0f - halff && x0 < halff)) {
        j1 = j0;
    }
}

// Share of the right pixel c+1 of a row segment whose left end is u, with
// fl = floor(u): (u - fl + |slope| - 1) / |slope| clamped to [0, 1].
__device__ __forceinline__ float right_share(float u, float fl, float ainv) {
    return __saturatef(__fmaf_rn(__fsub_rn(u, fl), ainv, __fsub_rn(1.0f, ainv)));
}

// ---------------------------------------------------------------------------
// Forward projection of one ray: sum over the rows of the traversal frame.
// img points at the image seen in that frame (the transposed image for flat
// lines).  ONES replaces every in-bounds pixel by 1 (normaliser R, FP64 sum).
// ---------------------------------------------------------------------------
template <bool ONES>
struct FpAcc;
template <> struct FpAcc<false> { typedef float T; };
template <> struct FpAcc<true> { typedef double T; };

// Rows [j0, j1) of the fast path, accumulated into (sum, comp): partial sums
// over 32 rows, compensated across partials.
template <bool ONES>
__device__ __forceinline__ void fp_rows_fast(const float *__restrict__ img, int N, float slope, float x0,
                                             float ainv, int j0, int j1,
                                             typename FpAcc<ONES>::T &sum, float &comp) {
    const unsigned uN = (unsigned)N;
    const int half = N / 2;
    int j = j0;
    while (j < j1) {
        const int jend = min(j + 32, j1);
        float part = 0.0f;
        const float *row = img + (size_t)j * N;
#pragma unroll 4
        for (; j < jend; ++j, row += N) {
            // x = left end of the row segment, centred; c = its pixel index
            const float x = fmaf((float)(j - half), slope, x0);
            int c;
            const float fl = floor_magic(x, c);
            c += half;
            const float t = right_share(x, fl, ainv);                      // share of pixel c+1
            float v0, v1;
            if constexpr (ONES) {
                v0 = ((unsigned)c < uN) ? 1.0f : 0.0f;
                v1 = ((unsigned)(c + 1) < uN) ? 1.0f : 0.0f;
            } else {
                v0 = ((unsigned)c < uN) ? __ldg(row + c) : 0.0f;
                v1 = ((unsigned)(c + 1) < uN) ? __ldg(row + c + 1) : 0.0f;
            }
            part += fmaf(t, v1 - v0, v0);
        }
        if constexpr (ONES) sum += (double)part;
        else comp_add(sum, comp, part);
    }
}

// One frame row of the reference's own expressions (forwardprojection.fut:
// 32-56), used for near-axis lines: every operation rounds exactly as the f32
// reference.  Row i is centred (i in [-half, half)); img points at pixel (0, 0)
// of the frame, rows `stride` floats apart, pixels ESTEP floats apart (2: the
// first halves of a pair image).  When the segment stays in one
// pixel the reference's two quotients are not used (lines 47, 54), so they are
// only evaluated for two-pixel rows (xdiff can be 0 for an axis-parallel ray).
template <bool ONES, int ESTEP = 1>
__device__ __forceinline__ float fp_row_exact(const float *__restrict__ img, int stride, int half, float slope,
                                              float intercept, float lbase, int i) {
    const float xbot = __fadd_rn(__fmul_rn((float)i, slope), intercept);
    const float xtop = __fadd_rn(xbot, slope);
    const int xpb = (int)floorf(xbot);
    const int xpt = (int)floorf(xtop);
    const bool single = xpb == xpt;
    const bool botin = xpb >= -half && xpb < half;
    const bool topin = (!single) && xpt >= -half && xpt < half;
    float lxbot = lbase, lxtop = 0.0f;
    if (!single) {
        const float xpmax = (float)max(xpb, xpt);
        const float xdiff = __fsub_rn(xtop, xbot);
        lxbot = __fmul_rn(__fdiv_rn(__fsub_rn(xpmax, xbot), xdiff), lbase);
        lxtop = __fmul_rn(__fdiv_rn(__fsub_rn(xtop, xpmax), xdiff), lbase);
    }
    float bot = 0.0f, top = 0.0f;
    if constexpr (ONES) {
        if (botin) bot = lxbot;
        if (topin) top = lxtop;
    } else {
        const float *row = img + (size_t)(i + half) * stride + half * ESTEP;
        if (botin) bot = __fmul_rn(lxbot, __ldg(row + xpb * ESTEP));
        if (topin) top = __fmul_rn(lxtop, __ldg(row + xpt * ESTEP));
    }
    return __fadd_rn(bot, top);
}

// All rows of a near-axis line, in the reference's order.
template <bool ONES>
__device__ __forceinline__ void fp_rows_exact(const float *__restrict__ img, int stride, int half, float slope,
                                              float intercept, float lbase,
                                              typename FpAcc<ONES>::T &sum) {
    typename FpAcc<ONES>::T acc = 0;
    for (int i = -half; i < half; ++i)
        acc += (typename FpAcc<ONES>::T)fp_row_exact<ONES>(img, stride, half, slope, intercept, lbase, i);
    sum = acc;
}

// Ray sum of detector r of the angle with geometry g.  Returns the reference
// value sum_rows(lbot*img[bot] + ltop*img[top]) (lbase already applied).
template <bool ONES>
__device__ __forceinline__ typename FpAcc<ONES>::T fp_ray(const ProbGeom &P, const AngleGeom &g,
                                                          const float *__restrict__ img_frame, int r,
                                                          int jbeg, int jend) {
    typedef typename FpAcc<ONES>::T T;
    const float rho = __fadd_rn(P.rhozero, __fmul_rn((float)r, P.deltarho));   // forwardprojection.fut:28
    const float intercept = __fdiv_rn(rho, g.cost);                               // forwardprojection.fut:29
    // |rho| of any point of the image is at most N/sqrt(2): such a ray adds nothing
    if (fabsf(rho) > 0.75f * (float)P.N + 2.0f) return (T)0;
    if (g.exact) {
        // whole ray in one piece (only the row-part starting at 0 computes it)
        if (jbeg != 0) return (T)0;
        T s;
        fp_rows_exact<ONES>(img_frame, P.N, P.half, g.slope, intercept, g.lbase, s);   // unpadded frame
        return s;
    }
    // x(j) = xlo(row j) centred, xlo = xbot + min(slope,0), xbot = (j-half)*slope + intercept
    const float x0 = ray_x0(g, intercept);
    int j0, j1;
    ray_rows(P, g, x0, j0, j1);
    j0 = max(j0, jbeg);
    j1 = min(j1, jend);
    if (j1 < j0) j1 = j0;
    T sum = (T)0;
    float comp = 0.0f;
    fp_rows_fast<ONES>(img_frame, P.N, g.slope, x0, g.ainv, j0, j1, sum, comp);
    if (ONES) return sum * (double)g.lbase;
    return (T)(((float)sum + comp) * g.lbase);
}

// ---------------------------------------------------------------------------
// Backprojection of one pixel for one angle: sum over the candidate
// detectors.  Returns the contribution with lbase applied.
// ---------------------------------------------------------------------------
template <bool ONES>
__device__ __forceinline__ float bp_angle(const ProbGeom &P, const AngleGeom &g, const float *__restrict__ sino_row,
                                          int row, int col) {
    const int half = P.half;
    const int D = P.D;
    if (!g.exact) {
        const float xc = (float)(col - half) + 0.5f;
        const float yc = (float)(row - half) + 0.5f;
        const float rhoc = fmaf(xc, g.c, -yc * g.s);
        int s0;
        ceil_magic((rhoc - fact_f32() - P.rz_c) * P.inv_deltarho, s0);   // centred detector index
        float acc = 0.0f;
        float d = fmaf((float)s0, P.deltarho, P.rz_c) - rhoc;
        for (int q = 0; q < P.rpp; ++q, d += P.deltarho) {
            const int det = s0 + P.zi + q;
            const float w = __saturatef(fmaf(-fabsf(d), g.inv_b, g.h_over_b));
            if ((unsigned)det < (unsigned)D) acc = fmaf(w, ONES ? 1.0f : __ldg(sino_row + det), acc);
        }
        return acc * g.lbase;
    }
    // Near-axis line: the reference's own f32 expressions (backprojection.fut:46-64)
    // in the line's frame (flat lines see the transposed image, 75-77).
    const float xmin = (float)(g.flat ? row - half : col - half);
    const float ymin = (float)(g.flat ? col - half : row - half);
    const float fact = fact_f32();
    const float cost = g.cost, sint = g.sint;
    const float x = __fsub_rn(__fadd_rn(xmin, 0.5f), __fmul_rn(fact, cost));
    const float y = __fsub_rn(__fadd_rn(ymin, 0.5f), __fmul_rn(fact, sint));
    const float rho = __fadd_rn(__fmul_rn(cost, x), __fmul_rn(sint, y));
    const float s = ceilf(__fdiv_rn(__fsub_rn(rho, P.rhozero), P.deltarho));
    const float xbase = __fmul_rn(ymin, g.slope);
    float acc = 0.0f;
    for (int i = 0; i < P.rpp; ++i) {
        const float sprime = __fadd_rn(s, (float)i);
        const float r = __fadd_rn(__fmul_rn(sprime, P.deltarho), P.rhozero);
        const float xbot = __fadd_rn(xbase, __fdiv_rn(r, cost));
        const float xtop = __fadd_rn(xbot, g.slope);
        const float maxx = fmaxf(xbot, xtop), minx = fminf(xbot, xtop);
        // intersect_fact (backprojection.fut:22-33)
        const float lo = fmaxf(__fsub_rn(maxx, xmin), 0.0f);
        const float hi = fmaxf(__fsub_rn(__fadd_rn(xmin, 1.0f), minx), 0.0f);
        const float diff = __fsub_rn(maxx, minx);
        const float inside = fminf(lo, hi);
        // inside/0 is +inf in the reference, capped to 1 below
        const float prop = inside == 0.0f ? 0.0f : (diff == 0.0f ? 1.0f : __fdiv_rn(inside, diff));
        const float l = __fmul_rn(fminf(prop, 1.0f), g.lbase);
        const int det = (int)sprime;
        if (det >= 0 && det < D) acc = __fadd_rn(acc, __fmul_rn(l, ONES ? 1.0f : __ldg(sino_row + det)));
    }
    return acc;
}

__device__ __forceinline__ AngleGeom load_geom(const AngleGeom *__restrict__ gt, int k) {
    const float4 *p = reinterpret_cast<const float4 *>(gt + k);
    const float4 a = __ldg(p), b = __ldg(p + 1), c = __ldg(p + 2);
    AngleGeom g;
    g.cost = a.x; g.sint = a.y; g.lbase = a.z; g.slope = a.w;
    g.c = b.x; g.s = b.y; g.h_over_b = b.z; g.inv_b = b.w;
    g.slope_lo = c.x; g.ainv = c.y; g.flat = __float_as_int(c.z); g.exact = __float_as_int(c.w);
    return g;
}

// ---------------------------------------------------------------------------
// Kernel launchers implemented in the .cu files (all enqueue on `stream`).
// ---------------------------------------------------------------------------
struct AngleLists;
// SM count of the current device, queried once per device
int device_sms();

cudaError_t launch_geometry(const float *angles, int a, AngleGeom *geom, cudaStream_t stream);
cudaError_t launch_fp(const ProbGeom &P, const AngleLists &L, const float2 *xpair, const float2 *xTpair, float *sino,
                      cudaStream_t stream);
// scaled: scratch of 2*a*D floats for the lbase-scaled rows (faster inner
// loop; detector pairs on the dense in-range path), or null for the unscaled
// kernel (no scratch)
cudaError_t launch_bp(const ProbGeom &P, const AngleLists &L, const float *sino, float *img, cudaStream_t stream,
                      float *scaled);
// R, C and the lists of rays that only clip a corner pixel (their R stored
// negated; graze [4*capc] entries {k, r} by corner in ray order, glen
// [4*capc] their chords, goff [5] the prefix offsets; graze_tmp / glen_tmp
// [4*capc] and gcnt [4] are scratch; see rownorm_kernel / graze_sort_kernel)
cudaError_t launch_normalisers(const ProbGeom &P, float *R, float *C, int2 *graze, float *glen, int *goff,
                               int2 *graze_tmp, float *glen_tmp, int *gcnt, int capc, cudaStream_t stream);

// compare.cu: the validation programs (diff, mse, sanityCheck) in one pass.
typedef synk_compare_result CompareResult;
cudaError_t launch_compare(const float *sane, const float *test, long long n, float tol, CompareResult *out,
                           cudaStream_t stream);
// what: 0 = int32 count (diff), 1 = float32 sse/n (mse), 2 = uint8 all_ok (sanityCheck)
cudaError_t launch_compare_finish(const CompareResult *r, long long n, int what, void *dst, cudaStream_t stream);

}  // namespace synk

// Pixel-driven backprojection of a tile, shared by the standalone
// backprojector and the persistent SIRT kernel.
//
// A block of 256 threads owns a tile of 32 columns; thread (lane, warp) owns
// column lane and PIX rows spaced RSTEP apart.  The per-angle constants of
// the chord-length trapezoid are staged in shared memory 64 angles at a time
// and read as one broadcast float4 + one float per angle; each (pixel, angle)
// then costs ~16 FP32/INT instructions and two sinogram gathers:
//   q    = x_c*cos - y_c*sin - rhozero            (rho of the centre, shifted)
//   s0   = ceil((q - sqrt(2)/2) / deltarho)       (first candidate detector)
//   d_i  = s0*deltarho + i*deltarho - q           (signed distance ray -> centre)
//   w_i  = sat((h - |d_i|) / b)                   (chord / lbase)
//   acc += lbase * sum_i w_i * sino[k][s0 + i]
// which is the reference's per-pixel sum (backprojection.fut:48-65) with
// intersect_fact*lbase (22-33, 62) written as the exact chord length of the
// line through the unit pixel.  Near-axis angles (AngleGeom::exact) are staged
// with zero weight and summed afterwards with the reference's own expressions.
#pragma once

#include "synk_internal.cuh"

namespace synk {

constexpr int kBpChunk = 64;

struct BpStage {
    float4 cs[kBpChunk];   // cos, sin, h/b, 1/b
    float lb[kBpChunk];    // lbase
};

// Stages angles [k0, k0 + kBpChunk) of P (all threads of the block call it).
__device__ __forceinline__ void bp_stage(const ProbGeom &P, int k0, BpStage &st) {
    for (int i = threadIdx.x; i < kBpChunk; i += blockDim.x) {
        const int k = k0 + i;
        float4 v = make_float4(0.0f, 0.0f, -1.0f, 0.0f);   // zero weight
        float l = 0.0f;
        if (k < P.a) {
            const AngleGeom g = load_geom(P.geom, k);
            if (!g.exact) {
                v = make_float4(g.c, g.s, g.h_over_b, g.inv_b);
                l = g.lbase;
            }
        }
        st.cs[i] = v;
        st.lb[i] = l;
    }
}

// Accumulates angles k in [k0, k1) with (k - k0) % kstride == kphase of the
// staged chunk (chunk starts at kc) into acc[m] for the PIX pixels
// (row0 + m*RSTEP, col).  sino: the problem's sinogram [a][D].
template <int PIX, bool RPP2>
__device__ __forceinline__ void bp_chunk(const ProbGeom &P, const BpStage &st, int kc, int kend, int kphase,
                                         int kstride, const float *__restrict__ sino, float xc, float yc0,
                                         float ystep, float (&acc)[PIX]) {
    const float fact = fact_f32();
    const int D = P.D;
    const unsigned uD = (unsigned)D;
    const int nk = min(kBpChunk, kend - kc);
    for (int i = kphase; i < nk; i += kstride) {
        const float4 g = st.cs[i];
        const float lb = st.lb[i];
        const float *__restrict__ row = sino + (size_t)(kc + i) * D;
        // q for the first pixel, then step along the column
        float t = fmaf(-yc0, g.y, -P.rhozero);
        const float tstep = -ystep * g.y;
#pragma unroll
        for (int m = 0; m < PIX; ++m, t += tstep) {
            const float q = fmaf(xc, g.x, t);
            int s0;
            float s0f;
            if (RPP2) {
                s0f = ceil_magic(q - fact, s0);
            } else {
                s0f = ceil_magic((q - fact) * P.inv_deltarho, s0);
                s0f = s0f * P.deltarho;
            }
            float d = s0f - q;
            float a = 0.0f;
            if (RPP2) {
                const float w0 = __saturatef(fmaf(-fabsf(d), g.w, g.z));
                const float w1 = __saturatef(fmaf(-fabsf(d + 1.0f), g.w, g.z));
                const float v0 = ((unsigned)s0 < uD) ? __ldg(row + s0) : 0.0f;
                const float v1 = ((unsigned)(s0 + 1) < uD) ? __ldg(row + s0 + 1) : 0.0f;
                a = fmaf(w1, v1, w0 * v0);
            } else {
                for (int q2 = 0; q2 < P.rpp; ++q2, d += P.deltarho) {
                    const int det = s0 + q2;
                    const float w = __saturatef(fmaf(-fabsf(d), g.w, g.z));
                    if ((unsigned)det < uD) a = fmaf(w, __ldg(row + det), a);
                }
            }
            acc[m] = fmaf(lb, a, acc[m]);
        }
    }
}

// The near-axis angles of list[0..nexact) for the PIX pixels, the reference's
// own expressions (bp_angle's exact branch).
template <int PIX>
__device__ __forceinline__ void bp_exact_angles(const ProbGeom &P, const int *__restrict__ list, int nexact,
                                                int kphase, int kstride, const float *__restrict__ sino, int row0,
                                                int rstep, int col, float (&acc)[PIX]) {
    for (int e = kphase; e < nexact; e += kstride) {
        const int k = __ldg(list + e);
        const AngleGeom g = load_geom(P.geom, k);
#pragma unroll
        for (int m = 0; m < PIX; ++m) {
            const int row = row0 + m * rstep;
            if (row < P.N && col < P.N) acc[m] += bp_angle<false>(P, g, sino + (size_t)k * P.D, row, col);
        }
    }
}

cudaError_t launch_exact_list(const ProbGeom &P, int *list, int *count, cudaStream_t stream);

}  // namespace synk

// Pixel-driven backprojection of a tile, shared by the standalone
// backprojector and the persistent SIRT kernel.
//
// A block of 256 threads owns a tile of 32 columns; thread (lane, warp) owns
// column lane and PIX rows spaced RSTEP apart.  The per-angle constants of
// the chord-length trapezoid are staged in shared memory kBpChunk angles at a time
// and read as one broadcast float4 + one float2 per angle; each (pixel, angle)
// then costs ~14 FP32/INT instructions and two sinogram gathers:
//   q    = x_c*cos - y_c*sin - rz_c               (rho of the centre from the middle
//                                                  detector position rz_c, ProbGeom)
//   s0   = ceil((q - sqrt(2)/2) / deltarho) + zi  (first candidate detector)
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

// Angles per staged chunk (and per partial sum before the compensated
// total).  Fewer chunks mean fewer staging barriers; the whole angle set of a
// problem of up to 256 angles is one chunk.  SIRT at N=128 / 128 angles, 200
// iterations: 4.08 ms with 64, 3.96 with 128; N=256 / 180 angles: 8.73 ms with
// 128, 8.53 with 256; dense backprojection 4.09 / 4.07 / 4.05 ms with 64 /
// 128 / 256.
constexpr int kBpChunk = 256;

struct BpStage {
    float4 cs[kBpChunk];   // cos, sin, h/b, 1/b
    float2 le[kBpChunk];   // lbase, h/b - (1 - sqrt(2)/2)/b
};

// Stages angles [k0, k0 + kBpChunk) of P (all threads of the block call it).
__device__ __forceinline__ void bp_stage(const ProbGeom &P, int k0, BpStage &st) {
    for (int i = threadIdx.x; i < kBpChunk; i += blockDim.x) {
        const int k = k0 + i;
        float4 v = make_float4(0.0f, 0.0f, -1.0f, 0.0f);   // zero weight
        float2 l = make_float2(0.0f, -1.0f);
        if (k < P.a) {
            const AngleGeom g = load_geom(P.geom, k);
            if (!g.exact) {
                v = make_float4(g.c, g.s, g.h_over_b, g.inv_b);
                l = make_float2(g.lbase, fmaf(-(1.0f - fact_f32()), g.inv_b, g.h_over_b));
            }
        }
        st.cs[i] = v;
        st.le[i] = l;
    }
}

// Accumulates angles k in [kc, kend) with (k - kc) % kstride == kphase of the
// staged chunk into acc[m] for the PIX pixels (row0 + m*ystep, col) whose
// centres are (xc, yc0 + m*ystep).  sino: the problem's sinogram [a][D].
//
// UNIT (deltarho = 1): with q = rho_c - rz_c - sqrt(2)/2, the first
// candidate detector is ceil(q) + zi and e = ceil(q) - q is in [0, 1); the two
// candidates sit at signed distances e - sqrt(2)/2 and e + 1 - sqrt(2)/2
// from the centre (the second is never negative), so
//   w0 = sat(h/b - |e - sqrt(2)/2| / b),  w1 = sat(c1 - e/b),  c1 = h/b - (1 - sqrt(2)/2)/b.
// INRANGE: the host proved that every window [s0, s0+1] lies in [0, D).
// SCALED: the sinogram rows of the staged (non-near-axis) angles are already
// multiplied by their lbase (row_scale), which saves one multiply per
// (pixel, angle); near-axis rows stay unscaled for bp_exact_angles.
// UNR = 2 (4) walks the angles two (four) at a time, so that their gathers
// are in flight together; the sums stay in angle order, bit for bit those of
// UNR = 1.
// PAIR (INRANGE only): sino holds detector pairs, entry s of row k =
// (row[s], row[s+1]) at float offset 2*(k*D + s), so one 8-byte gather serves
// both candidates (the same values, the same sums).
// Measured on GB300: SIRT at N=128 6.20 -> 5.88 ms (200 iterations; few warps
// there hide the gathers' latency), the dense backprojector at N=2048 4.88 ->
// 4.73 ms.
template <int PIX, bool UNIT, bool INRANGE, bool SCALED, int UNR = 1, bool PAIR = false>
__device__ __forceinline__ void bp_chunk(const ProbGeom &P, const BpStage &st, int kc, int kend, int kphase,
                                         int kstride, const float *__restrict__ sino, float xc, float yc0,
                                         float ystep, float (&acc)[PIX]) {
    const float fact = fact_f32();
    const int D = P.D;
    const unsigned uD = (unsigned)D;
    const int nk = min(kBpChunk, kend - kc);
    const float zoff = -P.rz_c - fact;        // centred: |q| stays below ~N/sqrt(2) + 1
    // INRANGE gather base: row + zi - kMagicBits (the magic constant's bits folded in)
    static_assert(!PAIR || INRANGE, "pair rows only on the in-range path");
    const uintptr_t zoffb = (uintptr_t)(((intptr_t)P.zi - (intptr_t)kMagicBits) * (PAIR ? 8 : 4));
    auto angle = [&](int i) {
        const float4 g = st.cs[i];
        const float2 le = st.le[i];
        const float *__restrict__ row = sino + (size_t)(kc + i) * D * (PAIR ? 2 : 1);
        if constexpr (UNIT) {
            // q of pixel m from the angle's base value in one rounding
            // (fma(m, dq, q0)), not by repeated additions: those drift by up
            // to PIX-1 roundings of |q| ~ D/2, which near-axis-adjacent
            // angles (trapezoid edges 1/b steep) turn into visible weight errors
            const float q0 = fmaf(xc, g.x, fmaf(-yc0, g.y, zoff));
            const float dq = -ystep * g.y;
            // INRANGE: the address comes straight from the bits of the rounded
            // sum r = q + 1.5*2^23 (bits(r) = bits(1.5*2^23) + s0), that constant
            // folded into the row base: one wide multiply-add per gather pair
            const uintptr_t rowb = reinterpret_cast<uintptr_t>(row) + zoffb;
#pragma unroll
            for (int m = 0; m < PIX; ++m) {
                const float q = m ? fmaf((float)m, dq, q0) : q0;
                float v0, v1, e;
                if constexpr (INRANGE) {
                    const float r = __fadd_ru(q, kMagic);
                    e = __fsub_rn(r, kMagic) - q;
                    if constexpr (PAIR) {
                        const float2 v = __ldg(reinterpret_cast<const float2 *>(
                            rowb + (uintptr_t)(unsigned)__float_as_int(r) * 8u));
                        v0 = v.x;
                        v1 = v.y;
                    } else {
                        const float *p = reinterpret_cast<const float *>(
                            rowb + (uintptr_t)(unsigned)__float_as_int(r) * 4u);
                        v0 = __ldg(p);
                        v1 = __ldg(p + 1);
                    }
                } else {
                    int s0;
                    e = ceil_magic(q, s0) - q;
                    s0 += P.zi;
                    v0 = ((unsigned)s0 < uD) ? __ldg(row + s0) : 0.0f;
                    v1 = ((unsigned)(s0 + 1) < uD) ? __ldg(row + s0 + 1) : 0.0f;
                }
                const float w0 = __saturatef(fmaf(-fabsf(e - fact), g.w, g.z));
                const float w1 = __saturatef(fmaf(-e, g.w, le.y));
                if constexpr (SCALED) acc[m] = fmaf(w1, v1, fmaf(w0, v0, acc[m]));
                else acc[m] = fmaf(le.x, fmaf(w1, v1, w0 * v0), acc[m]);
            }
        } else {
            const float t0 = fmaf(-yc0, g.y, -P.rz_c);
            const float tstep = -ystep * g.y;
#pragma unroll
            for (int m = 0; m < PIX; ++m) {
                const float t = m ? fmaf((float)m, tstep, t0) : t0;
                const float qc = fmaf(xc, g.x, t);             // rho_c - rz_c
                int s0;
                float s0f = ceil_magic((qc - fact) * P.inv_deltarho, s0);
                float d = s0f * P.deltarho - qc;
                float a = 0.0f;
                for (int q2 = 0; q2 < P.rpp; ++q2, d += P.deltarho) {
                    const int det = s0 + P.zi + q2;
                    const float w = __saturatef(fmaf(-fabsf(d), g.w, g.z));
                    if ((unsigned)det < uD) a = fmaf(w, __ldg(row + det), a);
                }
                acc[m] = SCALED ? acc[m] + a : fmaf(le.x, a, acc[m]);
            }
        }
    };
    int i = kphase;
    if constexpr (UNR == 4)
        for (; i + 3 * kstride < nk; i += 4 * kstride) {
            angle(i);
            angle(i + kstride);
            angle(i + 2 * kstride);
            angle(i + 3 * kstride);
        }
    if constexpr (UNR >= 2)
        for (; i + kstride < nk; i += 2 * kstride) {
            angle(i);
            angle(i + kstride);
        }
    for (; i < nk; i += kstride) angle(i);
}

// Factor of sinogram row k in a SCALED backprojection: lbase, or 1 for a
// near-axis angle (summed from the unscaled row by bp_exact_angles).
__device__ __forceinline__ float row_scale(const AngleGeom *__restrict__ geom, int k) {
    return __ldg(&geom[k].exact) ? 1.0f : __ldg(&geom[k].lbase);
}

// True when every pixel's two candidate detectors of the UNIT path lie in
// [0, D) (deltarho = 1 and a detector row covering the image's circumcircle,
// as the reference's D >= ceil(N*sqrt(2)) with centred rhozero does).  The
// tiles cover columns [0, 32*ceil(N/32)) and rows [0, tile_rows*ceil(N/tile_rows))
// (pixels past N are computed, not stored), so the bound takes the padded
// extent, and it keeps a margin for the float rounding of q.  A launch whose
// tile height divides tile_rows never reaches further.
inline bool bp_windows_in_range(const ProbGeom &P, int tile_rows) {
    if (P.deltarho != 1.0f) return false;
    const int ext_x = (P.N + 31) / 32 * 32;
    const int ext_y = (P.N + tile_rows - 1) / tile_rows * tile_rows;
    const int ext = ext_x > ext_y ? ext_x : ext_y;
    const double m = fmax(P.half - 0.5, ext - 0.5 - P.half);       // max |x_c|, |y_c| of a tile pixel
    const double R = m * 1.4142135623730951;                         // max |rho_c|
    const double f = 0.70710677;
    const double rz = (double)P.rhozero;
    const double margin = 1e-2 + 1e-5 * (R + fabs(rz));
    const double lo = -R - f - rz, hi = R - f - rz;
    return ceil(lo - margin) >= 0.0 && ceil(hi + margin) + 1.0 <= (double)P.D - 1.0;
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

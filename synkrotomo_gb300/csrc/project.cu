// Projector kernels of libsynk: per-angle geometry table, angle lists,
// padded/transposed and pair image copies, the forward projector
// (futhark/forwardprojection.fut:21-84), the backprojector
// (futhark/backprojection.fut:19-93) and the SIRT normalisers
// R = 1/(A*1), C = 1/(A^T*1) (futhark/SIRT.fut:22-25).
//
//   setup:    setup_kernel     geometry table + angle lists (+ pair images), one launch
//   forward:  fp_lane_kernel   8 detectors x 32 angles of one class per block
//                              (4 angles x 8 detectors per warp; with row parts
//                              one detector x 32 angles per warp)
//             fp_det_kernel    fewer than 32 angles: one warp = 32 detectors of one angle
//             fp_exact_kernel  near-axis angles, the reference's expressions
//   backward: bp_tile_kernel   one block = 32 x 8*PIX pixels, PIX = 4 or 8 per thread, all angles
//             bp_split_kernel  the same with the angles split over warps (images too small
//                              for one block per tile to fill the GPU)
// See fp_tile.cuh and bp_tile.cuh for the per-ray and per-pixel arithmetic.
#include <limits.h>
#include <math.h>

#include "synk_internal.cuh"
#include "fp_tile.cuh"
#include "bp_tile.cuh"

namespace synk {

int device_sms() {
    static int cache[64] = {0};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    if (!cache[dev]) {
        int sms = 0;
        if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) return 152;
        cache[dev] = sms;
    }
    return cache[dev];
}

// sirtlib.fut:28-44 per angle, plus the constants of both traversals.  cos
// and sin are evaluated in FP64 and rounded once, so they are the correctly
// rounded float32 values that the reference's f32.cos / f32.sin return for
// all practical inputs.
// Geometry table entry of angle theta (every kernel that builds the table
// uses this one function, so their tables are bit-identical).
__device__ __forceinline__ AngleGeom angle_geometry(float theta) {
    const double th = (double)theta;
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
    return g;
}

__global__ void geometry_kernel(const float *__restrict__ angles, int a, AngleGeom *__restrict__ geom) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= a) return;
    geom[k] = angle_geometry(angles[k]);
}

cudaError_t launch_geometry(const float *angles, int a, AngleGeom *geom, cudaStream_t stream) {
    geometry_kernel<<<(a + 127) / 128, 128, 0, stream>>>(angles, a, geom);
    return cudaGetLastError();
}

// Ordered compaction of the angles into: steep fast-path angles (padded with
// -1 to whole groups of 32), flat fast-path angles (padded likewise), and the
// near-axis angles.  One block; deterministic order (ascending angle index).
__global__ void __launch_bounds__(1024) angle_lists_kernel(const AngleGeom *__restrict__ geom, int a,
                                                           int *__restrict__ order, int *__restrict__ exact,
                                                           int *__restrict__ counts) {
    __shared__ int sh[1024];
    __shared__ int s_total;
    int base_order = 0;
    int nexact = 0;
    for (int cls = 0; cls < 3; ++cls) {      // 0 steep, 1 flat, 2 near-axis
        int base = 0;
        for (int k0 = 0; k0 < a; k0 += 1024) {
            const int k = k0 + threadIdx.x;
            int f = 0;
            if (k < a) {
                const int fl = __ldg(reinterpret_cast<const int *>(geom + k) + 10);
                const int ex = __ldg(reinterpret_cast<const int *>(geom + k) + 11);
                f = cls == 2 ? ex : (!ex && fl == cls);
            }
            sh[threadIdx.x] = f;
            __syncthreads();
            for (int off = 1; off < 1024; off <<= 1) {
                const int v = threadIdx.x >= off ? sh[threadIdx.x - off] : 0;
                __syncthreads();
                sh[threadIdx.x] += v;
                __syncthreads();
            }
            if (f) {
                const int pos = base + sh[threadIdx.x] - 1;
                if (cls == 2) exact[pos] = k;
                else order[base_order + pos] = k;
            }
            if (threadIdx.x == 1023) s_total = sh[1023];
            __syncthreads();
            base += s_total;
            __syncthreads();
        }
        if (cls < 2) {
            const int groups = (base + 31) / 32;
            for (int i = base + threadIdx.x; i < groups * 32; i += blockDim.x) order[base_order + i] = -1;
            if (threadIdx.x == 0) counts[cls] = groups;
            base_order += groups * 32;
        } else {
            nexact = base;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) counts[2] = nexact;
}

cudaError_t launch_angle_lists(const ProbGeom &P, int *order, int *exact, int *counts, cudaStream_t stream) {
    angle_lists_kernel<<<1, 1024, 0, stream>>>(P.geom, P.a, order, exact, counts);
    return cudaGetLastError();
}

// Pair images of the forward projector: xpair[r][i] = (p(r, i), p(r, i+1) - p(r, i))
// and xTpair[c][i] = (q(c, i), q(c, i+1) - q(c, i)) for i in [0, N+1] (row stride
// N+2; entry N+1 is (0, 0)), where p(r, i) = x[r][i-1] and q(c, i) = x[i-1][c]
// for i in [1, N], 0 otherwise: a row segment over pixels c, c+1 with share t
// of c+1 adds first + t * second of entry c+1 (the difference rounds once, here).
//
// One launch for everything a projection needs before its main kernel.
// Block 0 builds the geometry table (unless have_geom: the table is already
// written) and the angle lists of angle_lists_kernel (same layout and order)
// with warp ballots: pass 1 writes the table and counts the classes, pass 2
// re-reads the class flags and writes every angle at its ordered position.  Blocks 1.. (when x is given) write the pair images,
// one tile of 32 entries x 32 rows each, while block 0 works: xpair reads its
// two values straight from x (coalesced along i), xTpair goes through a tile
// of x rows bx-1 .. bx+31 so that its writes are coalesced too.
__global__ void __launch_bounds__(1024) setup_kernel(const float *__restrict__ angles, int a,
                                                     AngleGeom *__restrict__ geom, int *__restrict__ order,
                                                     int *__restrict__ exact, int *__restrict__ counts,
                                                     const float *__restrict__ x, float2 *__restrict__ xpair,
                                                     float2 *__restrict__ xTpair, int N, bool have_geom) {
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    if (blockIdx.x == 0) {
        __shared__ int tot[3];
        __shared__ int woff[3][32];
        __shared__ int ctot[3];
        if (tid < 3) tot[tid] = 0;
        __syncthreads();
        for (int k0 = 0; k0 < a; k0 += 1024) {                  // pass 1
            const int k = k0 + tid;
            int cls = 3;
            if (k < a) {
                if (have_geom) {
                    const int *gi = reinterpret_cast<const int *>(geom + k);
                    cls = gi[11] ? 2 : gi[10];                    // exact, flat
                } else {
                    const AngleGeom g = angle_geometry(angles[k]);
                    geom[k] = g;
                    cls = g.exact ? 2 : g.flat;
                }
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const unsigned b = __ballot_sync(0xffffffffu, cls == c);
                if (lane == 0 && b) atomicAdd(&tot[c], __popc(b));
            }
        }
        __syncthreads();
        const int gs = (tot[0] + 31) / 32, gf = (tot[1] + 31) / 32;
        const unsigned below = (1u << lane) - 1u;
        int base0 = 0, base1 = 0, base2 = 0;
        for (int k0 = 0; k0 < a; k0 += 1024) {                  // pass 2
            const int k = k0 + tid;
            int cls = 3;
            if (k < a) {
                const int *gi = reinterpret_cast<const int *>(geom + k);
                cls = gi[11] ? 2 : gi[10];                        // exact, flat
            }
            unsigned b[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) b[c] = __ballot_sync(0xffffffffu, cls == c);
            if (lane == 0) {
                woff[0][w] = __popc(b[0]);
                woff[1][w] = __popc(b[1]);
                woff[2][w] = __popc(b[2]);
            }
            __syncthreads();
            if (w < 3) {                                          // exclusive scan of the 32 warp counts
                const int v = woff[w][lane];
                int incl = v;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int t = __shfl_up_sync(0xffffffffu, incl, o);
                    if (lane >= o) incl += t;
                }
                woff[w][lane] = incl - v;
                if (lane == 31) ctot[w] = incl;
            }
            __syncthreads();
            if (cls == 0) order[base0 + woff[0][w] + __popc(b[0] & below)] = k;
            else if (cls == 1) order[gs * 32 + base1 + woff[1][w] + __popc(b[1] & below)] = k;
            else if (cls == 2) exact[base2 + woff[2][w] + __popc(b[2] & below)] = k;
            base0 += ctot[0];
            base1 += ctot[1];
            base2 += ctot[2];
            __syncthreads();
        }
        if (tid < 32) {
            if (tot[0] + tid < gs * 32) order[tot[0] + tid] = -1;
            if (tot[1] + tid < gf * 32) order[gs * 32 + tot[1] + tid] = -1;
        }
        if (tid == 0) {
            counts[0] = gs;
            counts[1] = gf;
            counts[2] = tot[2];
        }
        return;
    }
    // pair tiles: i in [bx, bx+32) of pair rows [by, by+32)
    __shared__ float tile[33][33];
    const int tiles_x = (N + 2 + 31) / 32;
    const int t = blockIdx.x - 1;
    const int bx = (t % tiles_x) * 32, by = (t / tiles_x) * 32;
    const int i = bx + lane;
    {
        const int r = by + w;
        if (r < N && i <= N + 1) {
            const float *xr = x + (size_t)r * N;
            const float va = (i >= 1 && i <= N) ? xr[i - 1] : 0.0f;
            const float vb = (i < N) ? xr[i] : 0.0f;
            xpair[(size_t)r * (N + 2) + i] = make_float2(va, __fsub_rn(vb, va));
        }
    }
    for (int y = w; y < 33; y += 32) {
        const int row = bx - 1 + y, c = by + lane;
        tile[y][lane] = (row >= 0 && row < N && c < N) ? x[(size_t)row * N + c] : 0.0f;
    }
    __syncthreads();
    const int c = by + w;
    if (c < N && i <= N + 1) {
        const float va = tile[lane][w];
        xTpair[(size_t)c * (N + 2) + i] = make_float2(va, __fsub_rn(tile[lane + 1][w], va));
    }
}

cudaError_t launch_setup(const float *angles, int a, AngleGeom *geom, int *order, int *exact, int *counts,
                         const float *x, float2 *xpair, float2 *xTpair, int N, cudaStream_t stream) {
    // Beyond one block's worth of angles the table's FP64 trigonometry is
    // spread over the geometry kernel's blocks first, and block 0 only reads
    // the class flags.
    const bool have_geom = a > 1024;
    if (have_geom) {
        cudaError_t e = launch_geometry(angles, a, geom, stream);
        if (e != cudaSuccess) return e;
    }
    const int tiles = x ? ((N + 2 + 31) / 32) * ((N + 31) / 32) : 0;
    setup_kernel<<<1 + tiles, 1024, 0, stream>>>(angles, a, geom, order, exact, counts, x, xpair, xTpair, N,
                                                 have_geom);
    return cudaGetLastError();
}

// xpad[z][r][c+1] = x[z][r][c], xTpad[z][c][r+1] = x[z][r][c] (row stride N+2);
// the blocks of the first and last tile column (row) also write the zero pad
// columns 0 and N+1 of their rows of xpad (xTpad).
__global__ void pad_kernel(const float *__restrict__ x, float *__restrict__ xpad, float *__restrict__ xTpad, int N) {
    __shared__ float tile[32][33];
    const size_t off = (size_t)blockIdx.z * N * N;
    const size_t offp = (size_t)blockIdx.z * N * (N + 2);
    const int bx = blockIdx.x * 32, by = blockIdx.y * 32;
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int r = by + y, c = bx + threadIdx.x;
        if (r < N && c < N) {
            const float v = x[off + (size_t)r * N + c];
            tile[y][threadIdx.x] = v;
            xpad[offp + (size_t)r * (N + 2) + c + 1] = v;
        }
    }
    if (threadIdx.y == 0 && (blockIdx.x == 0 || blockIdx.x == gridDim.x - 1)) {
        const int r = by + threadIdx.x;
        if (r < N) {
            if (blockIdx.x == 0) xpad[offp + (size_t)r * (N + 2)] = 0.0f;
            if (blockIdx.x == gridDim.x - 1) xpad[offp + (size_t)r * (N + 2) + N + 1] = 0.0f;
        }
    }
    if (threadIdx.y == 1 && (blockIdx.y == 0 || blockIdx.y == gridDim.y - 1)) {
        const int c = bx + threadIdx.x;
        if (c < N) {
            if (blockIdx.y == 0) xTpad[offp + (size_t)c * (N + 2)] = 0.0f;
            if (blockIdx.y == gridDim.y - 1) xTpad[offp + (size_t)c * (N + 2) + N + 1] = 0.0f;
        }
    }
    __syncthreads();
    for (int y = threadIdx.y; y < 32; y += 8) {
        const int c = bx + y, r = by + threadIdx.x;
        if (r < N && c < N) xTpad[offp + (size_t)c * (N + 2) + r + 1] = tile[threadIdx.x][y];
    }
}

cudaError_t launch_pad(const float *x, float *xpad, float *xTpad, int N, int nslices, cudaStream_t stream) {
    dim3 grid((N + 31) / 32, (N + 31) / 32, nslices);
    pad_kernel<<<grid, dim3(32, 8), 0, stream>>>(x, xpad, xTpad, N);
    return cudaGetLastError();
}

__global__ void unpad_kernel(const float *__restrict__ xpad, float *__restrict__ x, int N) {
    const size_t z = blockIdx.z;
    const int r = blockIdx.y;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < N; c += gridDim.x * blockDim.x)
        x[z * N * N + (size_t)r * N + c] = xpad[z * N * (N + 2) + (size_t)r * (N + 2) + c + 1];
}

cudaError_t launch_unpad(const float *xpad, float *x, int N, int nslices, cudaStream_t stream) {
    dim3 grid((N + 255) / 256, N, nslices);
    unpad_kernel<<<grid, 256, 0, stream>>>(xpad, x, N);
    return cudaGetLastError();
}

// ---- forward projection ---------------------------------------------------------

// A block = 8 warps = 8/S detectors x S row parts (S = 1, 2, 4, 8; with S = 1
// the block's 8 detectors x 32 angles are dealt 4 angles x 8 detectors per warp): with few
// angles (sparse-view data) the rays are split over rows so that enough warps
// are in flight; the S partial sums of a ray are added in a fixed order.
template <int S>
__global__ void __launch_bounds__(256) fp_lane_kernel(ProbGeom P, AngleLists L, const float2 *__restrict__ xpair,
                                                      const float2 *__restrict__ xTpair, float *__restrict__ sino) {
    __shared__ float red[8][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int grp = blockIdx.y;
    const int nsteep = __ldg(L.counts), nflat = __ldg(L.counts + 1);
    if (grp >= nsteep + nflat) return;              // block-uniform
    const int part = warp % S;
    int r, k;
    if (S == 1) {
        // the block's 8 detectors x 32 angles as 4 angles x 8 detectors per
        // warp: a warp's gathers of one row then span fewer sectors than with
        // 32 angles of one detector (FP at N=2048: 4.65 -> 4.53 ms; 8 x 4:
        // 4.58, 2 x 16: 4.61, 1 x 32: 4.68)
        r = blockIdx.x * 8 + (lane & 7);
        k = __ldg(L.order + grp * 32 + warp * 4 + (lane >> 3));
    } else {
        r = blockIdx.x * (8 / S) + warp / S;
        k = __ldg(L.order + grp * 32 + lane);
    }
    const int rr = r < P.D ? r : P.D - 1;          // keep every warp for the block reduction
    const int jb = part * P.N / S, je = (part + 1) * P.N / S;
    float v = fp_lane_ray_pair(P, r < P.D ? k : -1, rr, grp < nsteep ? xpair : xTpair, jb, je);
    if (S > 1) {
        red[warp][lane] = v;
        __syncthreads();
        if (part != 0) return;
        for (int t = 1; t < S; ++t) v += red[warp + t][lane];
    }
    if (k >= 0 && r < P.D) sino[(size_t)k * P.D + r] = v;
}

// Fewer than 32 angles (sparse-view data): one warp = 32 consecutive detectors
// of one angle, so no lane idles, and a block of 32 warps splits each ray into
// S row parts (S up to 32, at least 16 rows a part) so that each warp's chain
// of dependent gathers is short.  The per-ray arithmetic is fp_lane_kernel's
// (fp_lane_ray_pair); the S partial sums are added in a fixed order.
template <int S>
__global__ void __launch_bounds__(1024, 2) fp_det_kernel(ProbGeom P, AngleLists L, const float2 *__restrict__ xpair,
                                                      const float2 *__restrict__ xTpair, float *__restrict__ sino) {
    __shared__ float red[32][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int steep_slots = __ldg(L.counts) * 32;
    const int nslots = steep_slots + __ldg(L.counts + 1) * 32;
    const int slot = blockIdx.y;
    if (slot >= nslots) return;                       // block-uniform
    const int k = __ldg(L.order + slot);
    if (k < 0) return;                                // block-uniform: padding of a group
    const int part = warp % S;
    const int r = (blockIdx.x * (32 / S) + warp / S) * 32 + lane;
    const int jb = part * P.N / S, je = (part + 1) * P.N / S;
    const bool in = r < P.D;
    float v = fp_lane_ray_pair(P, in ? k : -1, in ? r : P.D - 1, slot < steep_slots ? xpair : xTpair, jb, je);
    if (S > 1) {
        red[warp][lane] = v;
        __syncthreads();
        if (part != 0) return;
        for (int t = 1; t < S; ++t) v += red[warp + t][lane];
    }
    if (in) sino[(size_t)k * P.D + r] = v;
}

// Near-axis rays (the reference's own expressions, on the pair images' first
// halves): a warp per (ray, row part), 8/S rays per block, kExactSlots angle
// slots (at most four near-axis angles lie in [0, 2 pi); repeats loop).
constexpr int kExactSlots = 4;

template <int S>
__global__ void __launch_bounds__(256) fp_exact_kernel(ProbGeom P, AngleLists L, const float2 *__restrict__ xpair,
                                                       const float2 *__restrict__ xTpair, float *__restrict__ sino) {
    __shared__ float red[8];
    const float *xpad = reinterpret_cast<const float *>(xpair);
    const float *xTpad = reinterpret_cast<const float *>(xTpair);
    const int nexact = __ldg(L.counts + 2);
    const int warp = threadIdx.x >> 5, part = warp % S;
    const int r = blockIdx.x * (8 / S) + warp / S;
    const int jb = part * P.N / S, je = (part + 1) * P.N / S;
    for (int e = blockIdx.y; e < nexact; e += gridDim.y) {      // block-uniform
        const int k = __ldg(L.exact + e);
        float v = r < P.D ? fp_exact_ray_warp<2>(P, k, r, xpad, xTpad, jb, je) : 0.0f;
        if (S > 1) {
            __syncthreads();
            if ((threadIdx.x & 31) == 0) red[warp] = v;
            __syncthreads();
            if (part == 0)
                for (int t = 1; t < S; ++t) v = __fadd_rn(v, red[warp + t]);
        }
        if (part == 0 && r < P.D && (threadIdx.x & 31) == 0) sino[(size_t)k * P.D + r] = v;
    }
}

// Rows split S ways when the rays alone give too few warps to fill the GPU.
static int fp_row_split(long long warps) {
    const int sms = device_sms();
    const long long want = (long long)sms * 48;
    int S = 1;
    while (S < 8 && warps * S < want) S *= 2;
    return S;
}

cudaError_t launch_fp(const ProbGeom &P, const AngleLists &L, const float2 *xpair, const float2 *xTpair, float *sino,
                      cudaStream_t stream) {
    if (P.a < 32) {
        // at most one group of each class: 64 angle slots; rows split to >= 16 a part
        int S = 1;
        while (S < 32 && P.N / (2 * S) >= 16) S *= 2;
        const int dgroups = (P.D + 31) / 32;
        const dim3 grid((dgroups + 32 / S - 1) / (32 / S), 64);
        switch (S) {
            case 1: fp_det_kernel<1><<<grid, 1024, 0, stream>>>(P, L, xpair, xTpair, sino); break;
            case 2: fp_det_kernel<2><<<grid, 1024, 0, stream>>>(P, L, xpair, xTpair, sino); break;
            case 4: fp_det_kernel<4><<<grid, 1024, 0, stream>>>(P, L, xpair, xTpair, sino); break;
            case 8: fp_det_kernel<8><<<grid, 1024, 0, stream>>>(P, L, xpair, xTpair, sino); break;
            case 16: fp_det_kernel<16><<<grid, 1024, 0, stream>>>(P, L, xpair, xTpair, sino); break;
            default: fp_det_kernel<32><<<grid, 1024, 0, stream>>>(P, L, xpair, xTpair, sino); break;
        }
    } else {
        // groups of 32 angles: at most ceil(a/32) + 2 (the steep/flat split adds one partial group each)
        const int gmax = (P.a + 31) / 32 + 2;
        const int S = fp_row_split((long long)((P.a + 31) / 32) * P.D);
        const dim3 grid((P.D + 8 / S - 1) / (8 / S), gmax);
        switch (S) {
            case 1: fp_lane_kernel<1><<<grid, 256, 0, stream>>>(P, L, xpair, xTpair, sino); break;
            case 2: fp_lane_kernel<2><<<grid, 256, 0, stream>>>(P, L, xpair, xTpair, sino); break;
            case 4: fp_lane_kernel<4><<<grid, 256, 0, stream>>>(P, L, xpair, xTpair, sino); break;
            default: fp_lane_kernel<8><<<grid, 256, 0, stream>>>(P, L, xpair, xTpair, sino); break;
        }
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    // near-axis angles: rays x angle slots must fill the GPU
    const int SE = fp_row_split((long long)P.D * 2);
    const dim3 ge((P.D + 8 / SE - 1) / (8 / SE), kExactSlots);
    switch (SE) {
        case 1: fp_exact_kernel<1><<<ge, 256, 0, stream>>>(P, L, xpair, xTpair, sino); break;
        case 2: fp_exact_kernel<2><<<ge, 256, 0, stream>>>(P, L, xpair, xTpair, sino); break;
        case 4: fp_exact_kernel<4><<<ge, 256, 0, stream>>>(P, L, xpair, xTpair, sino); break;
        default: fp_exact_kernel<8><<<ge, 256, 0, stream>>>(P, L, xpair, xTpair, sino); break;
    }
    return cudaGetLastError();
}

// ---- backprojection ---------------------------------------------------------------

// sino_s[k][r] = sino[k][r] * row_scale(k): the rows of a SCALED backprojection.
__global__ void __launch_bounds__(256) row_scale_kernel(ProbGeom P, const float *__restrict__ sino,
                                                        float *__restrict__ sino_s) {
    const int r = blockIdx.x * 256 + threadIdx.x;
    const int k = blockIdx.y;
    if (r >= P.D) return;
    const size_t i = (size_t)k * P.D + r;
    sino_s[i] = sino[i] * row_scale(P.geom, k);
}

// pair[k][s] = (v[s], v[s+1]) with v = sino[k] * row_scale(k) and v[D] = 0:
// the rows of a SCALED backprojection as detector pairs (bp_chunk's PAIR).
__global__ void __launch_bounds__(256) row_pair_kernel(ProbGeom P, const float *__restrict__ sino,
                                                       float2 *__restrict__ pair) {
    const int r = blockIdx.x * 256 + threadIdx.x;
    const int k = blockIdx.y;
    if (r >= P.D) return;
    const size_t i = (size_t)k * P.D + r;
    const float sc = row_scale(P.geom, k);
    const float v1 = r + 1 < P.D ? sino[i + 1] * sc : 0.0f;
    pair[i] = make_float2(sino[i] * sc, v1);
}

// Pixels per thread of the standalone backprojector (rows 8 apart: a block
// covers 32 columns x 8*PIX rows), and the resident blocks per SM each variant
// is compiled for.  8 pixels halve the per-angle overhead (dense data: 4.80 ms
// against 5.02 at N = 2048, 2048 angles); 4 give twice the blocks, which the
// few-angle (sparse-view) calls need.
template <int PIX>
struct BpShape {
    static constexpr int kMinBlocks = PIX == 8 ? 5 : 6;
};
constexpr int kBpManyAngles = 256;     // angle count from which the 8-pixel variant runs

// sino_s: the fast-path rows (scaled when SCALED, else sino itself); sino:
// the unscaled rows read by the near-axis angles.
// PAIR (the dense in-range path) walks the angles four at a time with 64
// registers (4 blocks per SM): 4.52 -> 4.14 ms at N = 2048, 2048 angles
// (two at a time with 48 registers and 5 blocks: 4.52; two with 64: 4.33).
template <int kBpPix, bool UNIT, bool INRANGE, bool SCALED, bool PAIR = false>
__global__ void __launch_bounds__(256, PAIR ? 4 : BpShape<kBpPix>::kMinBlocks) bp_tile_kernel(ProbGeom P, AngleLists L,
                                                                   const float *__restrict__ sino_s,
                                                                   const float *__restrict__ sino,
                                                                   float *__restrict__ out) {
    __shared__ BpStage st;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // PAIR: a warp's lanes are 8 columns x 4 rows of the tile (rows 8 apart per
    // pixel m as before), so one angle's gathers of a warp span fewer
    // detectors than 32 columns of one row (4.15 -> 4.09 ms; 16 x 2: 4.11)
    const int col = PAIR ? blockIdx.x * 32 + (warp & 3) * 8 + (lane & 7) : blockIdx.x * 32 + lane;
    const int row0 = PAIR ? blockIdx.y * (8 * kBpPix) + (warp >> 2) * 4 + (lane >> 3)
                          : blockIdx.y * (8 * kBpPix) + warp;
    const float xc = (float)(col - P.half) + 0.5f;
    const float yc0 = (float)(row0 - P.half) + 0.5f;
    float sum[kBpPix], comp[kBpPix];
#pragma unroll
    for (int m = 0; m < kBpPix; ++m) sum[m] = comp[m] = 0.0f;
    for (int kc = 0; kc < P.a; kc += kBpChunk) {
        __syncthreads();
        bp_stage(P, kc, st);
        __syncthreads();
        float part[kBpPix];
#pragma unroll
        for (int m = 0; m < kBpPix; ++m) part[m] = 0.0f;
        bp_chunk<kBpPix, UNIT, INRANGE, SCALED, PAIR ? 4 : 2, PAIR>(P, st, kc, P.a, 0, 1, sino_s, xc, yc0, 8.0f, part);
#pragma unroll
        for (int m = 0; m < kBpPix; ++m) comp_add(sum[m], comp[m], part[m]);
    }
    float ex[kBpPix];
#pragma unroll
    for (int m = 0; m < kBpPix; ++m) ex[m] = 0.0f;
    bp_exact_angles<kBpPix>(P, L.exact, __ldg(L.counts + 2), 0, 1, sino, row0, 8, col, ex);
#pragma unroll
    for (int m = 0; m < kBpPix; ++m) {
        const int row = row0 + 8 * m;
        if (row < P.N && col < P.N) out[(size_t)row * P.N + col] = (sum[m] + comp[m]) + ex[m];
    }
}

// The same pixels with the angles split SB ways (SB = 2, 4, 8), for images
// whose 32 x 8*PIX tiles are too few to fill the GPU: a block = 8/SB warp
// rows x SB angle parts, 32 x (8/SB)*PIX pixels; the SB partial sums of a
// pixel are added in a fixed order through shared memory.
template <int kBpPix, bool UNIT, bool INRANGE, bool SCALED>
__global__ void __launch_bounds__(256, BpShape<kBpPix>::kMinBlocks) bp_split_kernel(ProbGeom P, AngleLists L,
                                                                    const float *__restrict__ sino_s,
                                                                    const float *__restrict__ sino,
                                                                    float *__restrict__ out, int SB) {
    __shared__ BpStage st;
    __shared__ float red[8][kBpPix][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int RB = 8 / SB;
    const int part = warp % SB, wrow = warp / SB;
    const int col = blockIdx.x * 32 + lane;
    const int row0 = blockIdx.y * (RB * kBpPix) + wrow;
    const float xc = (float)(col - P.half) + 0.5f;
    const float yc0 = (float)(row0 - P.half) + 0.5f;
    float sum[kBpPix], comp[kBpPix];
#pragma unroll
    for (int m = 0; m < kBpPix; ++m) sum[m] = comp[m] = 0.0f;
    for (int kc = 0; kc < P.a; kc += kBpChunk) {
        __syncthreads();
        bp_stage(P, kc, st);
        __syncthreads();
        float prt[kBpPix];
#pragma unroll
        for (int m = 0; m < kBpPix; ++m) prt[m] = 0.0f;
        bp_chunk<kBpPix, UNIT, INRANGE, SCALED, 2>(P, st, kc, P.a, part, SB, sino_s, xc, yc0, (float)RB, prt);
#pragma unroll
        for (int m = 0; m < kBpPix; ++m) comp_add(sum[m], comp[m], prt[m]);
    }
    float ex[kBpPix];
#pragma unroll
    for (int m = 0; m < kBpPix; ++m) ex[m] = 0.0f;
    bp_exact_angles<kBpPix>(P, L.exact, __ldg(L.counts + 2), part, SB, sino, row0, RB, col, ex);
#pragma unroll
    for (int m = 0; m < kBpPix; ++m) red[warp][m][lane] = (sum[m] + comp[m]) + ex[m];
    __syncthreads();
    if (part != 0) return;
#pragma unroll
    for (int m = 0; m < kBpPix; ++m) {
        float v = red[warp][m][lane];
        for (int t = 1; t < SB; ++t) v += red[warp + t][m][lane];
        const int row = row0 + RB * m;
        if (row < P.N && col < P.N) out[(size_t)row * P.N + col] = v;
    }
}

// Angle split of the backprojection: the smallest SB whose tiles give at
// least four blocks per SM (1 when the unsplit tiles already do), with at
// least 8 angles per part (a split of a few angles only idles warps).
static int bp_angle_split(const ProbGeom &P, int pix) {
    const long long want = 4LL * device_sms();
    const long long cols = (P.N + 31) / 32;
    const int maxs = P.a >= 64 ? 8 : (P.a >= 32 ? 4 : (P.a >= 16 ? 2 : 1));
    int SB = 1;
    while (SB < maxs && cols * ((P.N + (8 / SB) * pix - 1) / ((8 / SB) * pix)) < want) SB *= 2;
    return SB;
}

template <int PIX, bool SCALED>
static void launch_bp_pix(const ProbGeom &P, const AngleLists &L, const float *sino_s, const float *sino, float *img,
                          cudaStream_t stream) {
    const int SB = bp_angle_split(P, PIX);
    const bool inrange = bp_windows_in_range(P, 8 * PIX);    // split tiles (8/SB)*PIX rows high divide 8*PIX
    const bool unit = P.deltarho == 1.0f;
    if (SB == 1) {
        const dim3 grid((P.N + 31) / 32, (P.N + 8 * PIX - 1) / (8 * PIX));
        if (inrange) bp_tile_kernel<PIX, true, true, SCALED><<<grid, 256, 0, stream>>>(P, L, sino_s, sino, img);
        else if (unit) bp_tile_kernel<PIX, true, false, SCALED><<<grid, 256, 0, stream>>>(P, L, sino_s, sino, img);
        else bp_tile_kernel<PIX, false, false, SCALED><<<grid, 256, 0, stream>>>(P, L, sino_s, sino, img);
    } else {
        const int th = (8 / SB) * PIX;
        const dim3 grid((P.N + 31) / 32, (P.N + th - 1) / th);
        if (inrange) bp_split_kernel<PIX, true, true, SCALED><<<grid, 256, 0, stream>>>(P, L, sino_s, sino, img, SB);
        else if (unit) bp_split_kernel<PIX, true, false, SCALED><<<grid, 256, 0, stream>>>(P, L, sino_s, sino, img, SB);
        else bp_split_kernel<PIX, false, false, SCALED><<<grid, 256, 0, stream>>>(P, L, sino_s, sino, img, SB);
    }
}

cudaError_t launch_bp(const ProbGeom &P, const AngleLists &L, const float *sino, float *img, cudaStream_t stream,
                      float *scaled) {
    if (scaled && P.a >= kBpManyAngles && bp_angle_split(P, 8) == 1 && bp_windows_in_range(P, 64)) {
        // dense data: detector pairs, one 8-byte gather per (pixel, angle)
        row_pair_kernel<<<dim3((P.D + 255) / 256, P.a), 256, 0, stream>>>(P, sino, reinterpret_cast<float2 *>(scaled));
        const dim3 grid((P.N + 31) / 32, (P.N + 63) / 64);
        bp_tile_kernel<8, true, true, true, true><<<grid, 256, 0, stream>>>(P, L, scaled, sino, img);
    } else if (scaled) {
        row_scale_kernel<<<dim3((P.D + 255) / 256, P.a), 256, 0, stream>>>(P, sino, scaled);
        if (P.a >= kBpManyAngles) launch_bp_pix<8, true>(P, L, scaled, sino, img, stream);
        else launch_bp_pix<4, true>(P, L, scaled, sino, img, stream);
    } else {
        if (P.a >= kBpManyAngles) launch_bp_pix<8, false>(P, L, sino, sino, img, stream);
        else launch_bp_pix<4, false>(P, L, sino, sino, img, stream);
    }
    return cudaGetLastError();
}

// ---- normalisers (FP64 sums) -----------------------------------------------------------

// The corner pixel a ray that only clips a corner cuts: the corner of the
// image square with the extreme rho = x cos - y sin on the ray's side
// (x = +-half at columns N-1 / 0, y = +-half at rows N-1 / 0); 0: row 0 col 0,
// 1: row 0 col N-1, 2: row N-1 col 0, 3: row N-1 col N-1.
__device__ __forceinline__ int graze_corner(const AngleGeom &g, float rho) {
    const bool right = (rho > 0.0f) == (g.c > 0.0f);
    const bool bottom = (rho > 0.0f) == (g.s < 0.0f);
    return (bottom ? 2 : 0) + (right ? 1 : 0);
}

// R = safe_inverse(A*1): one thread per ray (SIRT.fut:22-23, sirtlib.fut:9-13).
// A ray whose chord is under 1 cuts off a corner of the image inside one
// corner pixel.  There R = 1/chord magnifies the chord's rounding (the fast
// row rule and the backprojector's trapezoid differ by up to a few per cent
// on such rays), so the chord is the reference's own f32 sum
// (forwardprojection.fut:31-56), which equals the reference's backprojection
// weight for that pixel bit for bit.  Such a ray (of a fast-path angle;
// near-axis angles take the exact path anyway) is appended to its corner's
// list (graze, glen: unsorted, slots taken by atomics; graze_sort_kernel
// orders them) and its R is stored negated, which sends it to the SIRT
// kernels' exact treatment (sirt.cu).  A ray without a slot (not reached with
// the caller's bound) keeps the fast path.
__global__ void __launch_bounds__(256) rownorm_kernel(ProbGeom P, float *__restrict__ R, int2 *__restrict__ graze,
                                                      float *__restrict__ glen, int *__restrict__ gcnt, int capc) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int k = blockIdx.y * 8 + warp;
    const int r = blockIdx.x * 32 + lane;
    if (k >= P.a || r >= P.D) return;
    const AngleGeom g = load_geom(P.geom, k);
    const double v = fp_ray<true>(P, g, nullptr, r, 0, P.N);
    float Rv = v != 0.0 ? (float)(1.0 / v) : 0.0f;
    if (v > 0.0 && v < 1.0 && !g.exact) {
        const float e = fp_ray_exact_f32<true>(P, g, nullptr, 0, r);
        if (e != 0.0f) {
            const int c = graze_corner(g, __fadd_rn(P.rhozero, __fmul_rn((float)r, P.deltarho)));
            const int slot = atomicAdd(gcnt + c, 1);
            if (slot < capc) {
                graze[(size_t)c * capc + slot] = make_int2(k, r);
                glen[(size_t)c * capc + slot] = e;
                Rv = -__fdiv_rn(1.0f, e);
            }
        }
    }
    R[(size_t)k * P.D + r] = Rv;
}

// Orders each corner's list by ray (k, r) -- one block; a rank sort, each
// entry's position being the number of smaller keys -- into graze/glen, so
// every later sum over a list is deterministic; goff[0..4] are the prefix
// offsets of the flat order the SIRT forward items walk (corner c holds
// goff[c+1] - goff[c] entries).
__global__ void __launch_bounds__(1024) graze_sort_kernel(const int2 *__restrict__ ug, const float *__restrict__ ul,
                                                          const int *__restrict__ gcnt, int2 *__restrict__ graze,
                                                          float *__restrict__ glen, int *__restrict__ goff, int capc) {
    __shared__ int2 sh[1024];
    for (int c = 0; c < 4; ++c) {
        const int n = min(gcnt[c], capc);                  // block-uniform
        const int2 *u = ug + (size_t)c * capc;
        for (int i0 = 0; i0 < n; i0 += 1024) {
            const int i = i0 + (int)threadIdx.x;
            const int2 me = i < n ? u[i] : make_int2(INT_MAX, INT_MAX);
            int rank = 0;
            for (int j0 = 0; j0 < n; j0 += 1024) {
                __syncthreads();
                if (j0 + (int)threadIdx.x < n) sh[threadIdx.x] = u[j0 + threadIdx.x];
                __syncthreads();
                const int m = min(1024, n - j0);
                for (int j = 0; j < m; ++j) {
                    const int2 o = sh[j];
                    rank += (o.x < me.x || (o.x == me.x && o.y < me.y)) ? 1 : 0;
                }
            }
            if (i < n) {
                graze[(size_t)c * capc + rank] = me;
                glen[(size_t)c * capc + rank] = ul[(size_t)c * capc + i];
            }
        }
    }
    if (threadIdx.x == 0) {
        int o = 0;
        for (int c = 0; c < 4; ++c) {
            goff[c] = o;
            o += min(gcnt[c], capc);
        }
        goff[4] = o;
    }
}

// C = safe_inverse(A^T*1): one thread per pixel, FP64 angle sum (SIRT.fut:25).
__global__ void __launch_bounds__(256) colnorm_kernel(ProbGeom P, float *__restrict__ C) {
    const int col = blockIdx.x * 32 + (threadIdx.x & 31);
    const int row = blockIdx.y * 8 + (threadIdx.x >> 5);
    if (row >= P.N || col >= P.N) return;
    double dsum = 0.0;
    for (int k0 = 0; k0 < P.a; k0 += 32) {
        const int k1 = min(k0 + 32, P.a);
        float part = 0.0f;
        for (int k = k0; k < k1; ++k) part += bp_angle<true>(P, load_geom(P.geom, k), nullptr, row, col);
        dsum += (double)part;
    }
    C[(size_t)row * P.N + col] = dsum != 0.0 ? (float)(1.0 / dsum) : 0.0f;
}

cudaError_t launch_normalisers(const ProbGeom &P, float *R, float *C, int2 *graze, float *glen, int *goff,
                               int2 *graze_tmp, float *glen_tmp, int *gcnt, int capc, cudaStream_t stream) {
    cudaError_t e = cudaMemsetAsync(gcnt, 0, 4 * sizeof(int), stream);
    if (e != cudaSuccess) return e;
    dim3 gf((P.D + 31) / 32, (P.a + 7) / 8);
    rownorm_kernel<<<gf, 256, 0, stream>>>(P, R, graze_tmp, glen_tmp, gcnt, capc);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    graze_sort_kernel<<<1, 1024, 0, stream>>>(graze_tmp, glen_tmp, gcnt, graze, glen, goff, capc);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    dim3 gb((P.N + 31) / 32, (P.N + 7) / 8);
    colnorm_kernel<<<gb, 256, 0, stream>>>(P, C);
    return cudaGetLastError();
}

}  // namespace synk

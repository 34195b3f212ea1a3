// BF16 tensor-core GEMM engine on tcgen05 (sm_103a) for the U-Net warm
// starter: C[M x N] = A[M x K] * B[N x K]^T with FP32 accumulation in TMEM.
//
// One CTA = 6 warps and one 128-row tile of C with all N (<= 256) columns:
//   warp 0      TMA producer: per K chunk one A box and one B box into a
//               shared-memory stage (canonical K-major swizzled layout),
//               completion counted on the stage's "full" mbarrier
//   warp 1      MMA issuer (one thread): tcgen05.mma kind::f16 per 16-wide K
//               step, tcgen05.commit frees the stage ("empty" mbarrier), a last
//               commit signals the accumulator
//   warps 2-5   epilogue: tcgen05.ld of their 32 TMEM lanes, fused bias / ReLU /
//               ReLU-mask / atomic accumulation, stores
// Operand modes (how the producer addresses A and B):
//   MODE_GEMM   plain 2-D tensors (validation of the engine)
//   MODE_CONV   implicit-GEMM 3x3 convolution, pad 1, NHWC BF16: K = 9 taps x
//               input channels in chunks of 64 (128-byte rows, 128-byte
//               swizzle) when Cin allows, else 32; the A box of a tap is the
//               tile's 128 pixels shifted by the tap, read from a 4-D map
//               (C, W, H, batch) whose out-of-bounds zeros are the padding.
//               The backward-data pass is the same convolution of the output
//               gradient with the tap-flipped, transposed weights.
//   MODE_WGRAD  weight gradient: K = pixels, 64 (or 32) per chunk, of blocked
//               copies [image][row][pixel chunk][channel][pixel]; A = dY
//               (output channels), B = X shifted by the tap (three copies
//               pre-shifted along W; the H shift is the TMA coordinate), split
//               over K across CTAs with FP32 atomics.
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include "synk_internal.cuh"
#include "umma.cuh"
#include "umma_gemm.cuh"

namespace synk {
namespace unet {

using namespace umma;

__device__ __forceinline__ uint16_t f2bf(float x) {
    return __bfloat16_as_ushort(__float2bfloat16_rn(x));
}
__device__ __forceinline__ float bf2f(uint16_t x) { return __bfloat162float(__ushort_as_bfloat16(x)); }

// The coordinates of one output tile (linear index t over gx x gy x gz).
struct TileInfo {
    int m0, n0, kbeg, nk, b, h0, w0, ky, kx, tap;
};

template <int MODE>
__device__ __forceinline__ TileInfo tile_info(const GemmParams &p, long long t) {
    TileInfo ti = {};
    const int tx = (int)(t % p.gx);
    const long long r1 = t / p.gx;
    const int ty = (int)(r1 % p.gy);
    const int tz = (int)(r1 / p.gy);
    ti.n0 = ty * p.N;
    ti.nk = p.nk;
    if (MODE == MODE_GEMM) {
        ti.m0 = tx * 128;
    } else if (MODE == MODE_CONV || MODE == MODE_HALO) {
        const int tiles_w = p.W / p.bw, tpi = tiles_w * (p.H / p.bh);
        ti.b = tx / tpi;
        const int r = tx - ti.b * tpi;
        ti.h0 = (r / tiles_w) * p.bh;
        ti.w0 = (r - (r / tiles_w) * tiles_w) * p.bw;
    } else {   // MODE_WGRAD
        // taps vary fastest: the CTAs running at one time cover the nine taps of
        // the same pixel range, which then come from L2 instead of HBM
        ti.m0 = tx * 128;
        const int ks = tz / 9;
        ti.tap = tz - ks * 9;
        ti.ky = ti.tap / 3;
        ti.kx = ti.tap - ti.ky * 3;
        const long long nbk = (long long)p.Bn * p.nb_h * p.nb_w;
        ti.kbeg = (int)(nbk * ks / p.ksplit);
        ti.nk = (int)(nbk * (ks + 1) / p.ksplit) - ti.kbeg;
    }
    return ti;
}

// Persistent: one CTA per SM walks tiles t = blockIdx.x, += gridDim.x.  The
// shared-memory stage ring runs continuously across tiles, and the FP32
// accumulator is double-buffered in TMEM (2 x ncols columns): the MMA warp
// fills buffer (i & 1) for tile i while the epilogue warps drain the other.
//   full[s]   TMA -> MMA     (expect_tx bytes)       empty[s]  MMA -> TMA (tcgen05.commit)
//   tfull[j]  MMA -> epilogue (tcgen05.commit)       tempty[j] epilogue -> MMA (4 warp arrivals)
template <int MODE, int EPI>
__global__ void __launch_bounds__(192, 1) umma_kernel(const __grid_constant__ CUtensorMap tmA,
                                                      const __grid_constant__ CUtensorMap tmB, const GemmParams p) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    uint8_t *smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    // stage = A part + B part (sizes from the host; MODE_HALO: A = one 130-pixel
    // row strip of 128-byte rows, B = the 3 taps kx of the strip's ky)
    const uint32_t aBytes = p.aStage;
    const uint32_t bBytes = p.bStage;
    const uint32_t bTap = (uint32_t)p.N * 128u;        // MODE_HALO: one tap's weights
    const uint32_t stageBytes = aBytes + bBytes;
    const int S = p.stages;
    uint8_t *bres = smem + (size_t)S * stageBytes;      // resident B (MODE_HALO, p.bres > 0)
    uint64_t *full = reinterpret_cast<uint64_t *>(bres + p.bres);
    uint64_t *empty = full + S;
    uint64_t *tfull = empty + S;
    uint64_t *tempty = tfull + 2;
    uint64_t *drain = tempty + 2;
    uint64_t *bfull = drain + 1;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(bfull + 1);
    float *sbias = reinterpret_cast<float *>(tmem_slot + 4);    // [gy * N] epilogue bias

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        tmem_alloc(tmem_slot, 2u * (uint32_t)p.ncols);
        tmem_relinquish();
    }
    if (warp == 1 && lane == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        for (int j = 0; j < 2; ++j) {
            mbar_init(&tfull[j], 1);
            mbar_init(&tempty[j], 4);
        }
        mbar_init(drain, 1);
        mbar_init(bfull, 1);
        fence_mbar_init();
    }
    if (warp == 0 && lane == 0) {
        tma_prefetch_desc(&tmA);
        tma_prefetch_desc(&tmB);
    }
    if (EPI == EPI_BIAS_RELU || EPI == EPI_BIAS)
        for (int i = threadIdx.x; i < p.gy * p.N; i += blockDim.x) sbias[i] = p.bias[i];
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;
    const long long ntiles = p.ntiles;

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer ----
            long long g = 0;   // chunks issued by this CTA
            bool fail = false;
            if (MODE == MODE_HALO && p.bres) {
                // all taps' weights once for the CTA's lifetime (one n tile)
                mbar_arrive_expect_tx(bfull, p.bres);
                tma_load_3d(bres, &tmB, bfull, 0, 0, 0);
            }
            for (long long t = blockIdx.x; t < ntiles && !fail; t += gridDim.x) {
                const TileInfo ti = tile_info<MODE>(p, t);
                for (int kc = 0; kc < ti.nk; ++kc) {
                    const int s = (int)(g % S);
                    const uint32_t ph = (uint32_t)(g / S) & 1u;
                    if (g >= S && !mbar_wait(&empty[s], ph ^ 1u, p.err, p.limit_ns)) {
                        fail = true;
                        break;
                    }
                    uint8_t *As = smem + (size_t)s * stageBytes;
                    uint8_t *Bs = As + aBytes;
                    mbar_arrive_expect_tx(&full[s], p.bytesA + p.bytesB);
                    if (MODE == MODE_GEMM) {
                        const int ke = p.kbytes / 2;
                        tma_load_2d(As, &tmA, &full[s], kc * ke, ti.m0);
                        tma_load_2d(Bs, &tmB, &full[s], kc * ke, ti.n0);
                    } else if (MODE == MODE_HALO) {
                        // chunk = (ky, channel chunk cc): the strip of row h0+ky-1,
                        // pixels w0-1 .. w0+128, and the weights of taps (ky, 0..2)
                        // (64-channel boxes; channels >= Cin are out of bounds and read as 0)
                        // B: packed weights [chunk][tap][Cout][64]; the three taps of row ky
                        // are one box (few large TMA operations keep the copy engine busy)
                        const int ky = kc / p.cchunks, cc = kc - ky * p.cchunks;
                        tma_load_4d(As, &tmA, &full[s], cc * 64, ti.w0 - 1, ti.h0 + ky - 1, ti.b);
                        if (!p.bres) tma_load_3d(Bs, &tmB, &full[s], 0, ti.n0, cc * 9 + 3 * ky);
                    } else if (MODE == MODE_CONV) {
                        const int tap = kc / p.cchunks, cc = kc - tap * p.cchunks;
                        const int tky = tap / 3, tkx = tap - tky * 3;
                        const int cw = p.kbytes / 2;   // channels per chunk
                        tma_load_4d(As, &tmA, &full[s], cc * cw, ti.w0 + tkx - 1, ti.h0 + tky - 1, ti.b);
                        tma_load_2d(Bs, &tmB, &full[s], tap * p.Cin + cc * cw, ti.n0);
                    } else {
                        const int pb = ti.kbeg + kc;
                        const int per_img = p.nb_h * p.nb_w;
                        const int bb = pb / per_img;
                        const int r = pb - bb * per_img;
                        const int hb = r / p.nb_w, wb = r - (r / p.nb_w) * p.nb_w;
                        // blocked operands [image][row][pixel chunk][channel][pixel]: a box is
                        // one contiguous block; the tap's row shift is the H coordinate (zero
                        // outside the image) and its column shift the pre-shifted copy kx
                        // a stage holds kw x kh pixel chunks (one box per operand)
                        tma_load_5d(As, &tmA, &full[s], 0, ti.m0, wb * p.kw, hb * p.kh, bb);
                        tma_load_5d(Bs, &tmB, &full[s], 0, ti.n0, wb * p.kw, hb * p.kh + ti.ky - 1,
                                    ti.kx * p.Bn + bb);
                    }
                    ++g;
                }
            }
            // no copy may still be landing when the CTA exits: wait (bounded) for
            // the last use of every stage (immediate on the normal path)
            const long long first = g > S ? g - S : 0;
            for (long long c = first; c < g; ++c) mbar_drain(&full[c % S], (uint32_t)(c / S) & 1u, p.limit_ns);
            if (MODE == MODE_HALO && p.bres) mbar_drain(bfull, 0u, p.limit_ns);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer ----
            const uint32_t idesc = idesc_bf16(128, p.N);
            const uint32_t kbytes = (uint32_t)p.kbytes;
            long long g = 0;
            int li = 0;
            bool fail = false;
            if (MODE == MODE_HALO && p.bres && !mbar_wait(bfull, 0u, p.err, p.limit_ns)) fail = true;
            for (long long t = blockIdx.x; t < ntiles && !fail; t += gridDim.x, ++li) {
                const TileInfo ti = tile_info<MODE>(p, t);
                const int ab = li & 1;
                const uint32_t dt = tmem + (uint32_t)(ab * p.ncols);
                if (li >= 2 && !mbar_wait(&tempty[ab], (uint32_t)((li >> 1) - 1) & 1u, p.err, p.limit_ns)) break;
                tc_fence_after();
                for (int kc = 0; kc < ti.nk; ++kc, ++g) {
                    const int s = (int)(g % S);
                    const uint32_t ph = (uint32_t)(g / S) & 1u;
                    if (!mbar_wait(&full[s], ph, p.err, p.limit_ns)) {
                        fail = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t a0 = smem_u32(smem + (size_t)s * stageBytes);
                    const uint32_t b0 = a0 + aBytes;
                    if (MODE == MODE_HALO) {
                        // tap kx reads the strip from row kx (pixel w0+kx-1); only the
                        // chunk's valid channels (32 or 64) are multiplied
                        const int ky = kc / p.cchunks, cc = kc - ky * p.cchunks;
                        const uint32_t ksteps = (uint32_t)min(64, p.Cin - 64 * cc) / 16u;
                        // weights of tap (ky, kx): resident block (cc*9 + 3ky + kx) or the stage's box kx
                        const uint32_t bt0 = p.bres ? smem_u32(bres) + (uint32_t)(cc * 9 + 3 * ky) * bTap : b0;
                        for (uint32_t kx = 0; kx < 3u; ++kx)
                            for (uint32_t kk = 0; kk < ksteps; ++kk)
                                mma_bf16(dt, smem_desc_sw128_at(a0 + kx * 128u + kk * 32u),
                                         smem_desc(bt0 + kx * bTap + kk * 32u, 128u), idesc,
                                         (kc | (int)kx | (int)kk) != 0 ? 1u : 0u);
                    } else if (MODE == MODE_WGRAD) {
                        // sub-chunk j of the stage: A rows at j*arows, B rows at j*N
                        const uint32_t nsub = (uint32_t)(p.kw * p.kh);
                        for (uint32_t j = 0; j < nsub; ++j)
                            for (uint32_t kk = 0; kk < kbytes / 32u; ++kk)
                                mma_bf16(dt, smem_desc(a0 + j * (uint32_t)p.arows * kbytes + kk * 32u, kbytes),
                                         smem_desc(b0 + j * (uint32_t)p.N * kbytes + kk * 32u, kbytes), idesc,
                                         (kc | (int)j | (int)kk) != 0 ? 1u : 0u);
                    } else {
                        for (uint32_t kk = 0; kk < kbytes / 32u; ++kk) {
                            mma_bf16(dt, smem_desc(a0 + kk * 32u, kbytes), smem_desc(b0 + kk * 32u, kbytes), idesc,
                                     (kc | (int)kk) != 0 ? 1u : 0u);
                        }
                    }
                    mma_commit(&empty[s]);
                }
                if (!fail) mma_commit(&tfull[ab]);
            }
            // every issued MMA has completed before TMEM is freed
            mma_commit(drain);
            mbar_drain(drain, 0u, p.limit_ns);
        }
    } else {
        // ---- epilogue (warps 2..5): TMEM lanes 32*(warp % 4) .. +31 ----
        const int q = warp & 3;
        const int row = q * 32 + lane;
        int li = 0;
        for (long long t = blockIdx.x; t < ntiles; t += gridDim.x, ++li) {
            const TileInfo ti = tile_info<MODE>(p, t);
            const int ab = li & 1;
            const bool ok = mbar_wait(&tfull[ab], (uint32_t)(li >> 1) & 1u, p.err, p.limit_ns);
            tc_fence_after();
            // tcgen05.ld is warp-collective: decide once per warp
            const bool good = __all_sync(0xffffffffu, ok && *(volatile int *)p.err == 0);
            if (!good) break;
            // a split-K tile with no chunks contributes nothing (its buffer was not written)
            const int ncol = ti.nk > 0 ? p.N : 0;
            long long pix = 0;
            bool rvalid = true;
            if (MODE == MODE_GEMM) {
                rvalid = ti.m0 + row < p.M;
            } else if (MODE == MODE_CONV || MODE == MODE_HALO) {
                const int h = ti.h0 + row / p.bw, w = ti.w0 + (row - (row / p.bw) * p.bw);
                pix = ((long long)ti.b * p.H + h) * p.W + w;
            } else {
                rvalid = ti.m0 + row < p.mvalid;
            }
            const uint32_t tbase = tmem + (uint32_t)(ab * p.ncols) + ((uint32_t)(q * 32) << 16);
            for (int c0 = 0; c0 < ncol; c0 += 32) {
                float v[32];
                tmem_ld_32x32(tbase + (uint32_t)c0, v);
                if (!rvalid) continue;
                const int nbase = ti.n0 + c0;
                const int nval = min(32, p.N - c0);
                if (EPI == EPI_F32) {
                    float *o = reinterpret_cast<float *>(p.out) + (long long)(ti.m0 + row) * p.ldo + nbase;
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (j < nval) o[j] = v[j];
                } else if (EPI == EPI_ATOMIC) {
                    float *o = reinterpret_cast<float *>(p.out) + (long long)(ti.m0 + row) * p.ldo + ti.tap * p.Cin +
                               nbase;
                    const int lim = min(nval, p.Cin - nbase);
#pragma unroll
                    for (int j = 0; j < 32; ++j)
                        if (j < lim) atomicAdd(o + j, v[j]);
                } else {
                    uint16_t *o = reinterpret_cast<uint16_t *>(p.out) + pix * p.ldo + p.coff + nbase;
                    uint32_t pk[16];
                    uint32_t mw[16];
                    if (EPI == EPI_MASK) {
                        const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask + pix * p.ldm + p.moff + nbase);
#pragma unroll
                        for (int t4 = 0; t4 < 4; ++t4) {
                            const uint4 u = (t4 * 8 < nval) ? mk[t4] : make_uint4(0u, 0u, 0u, 0u);
                            mw[4 * t4] = u.x;
                            mw[4 * t4 + 1] = u.y;
                            mw[4 * t4 + 2] = u.z;
                            mw[4 * t4 + 3] = u.w;
                        }
                    }
#pragma unroll
                    for (int j = 0; j < 32; j += 2) {
                        float x0 = v[j], x1 = v[j + 1];
                        if (EPI == EPI_BIAS_RELU || EPI == EPI_BIAS) {
                            x0 += sbias[nbase + j];
                            x1 += sbias[nbase + j + 1];
                            if (EPI == EPI_BIAS_RELU) {
                                x0 = fmaxf(x0, 0.0f);
                                x1 = fmaxf(x1, 0.0f);
                            }
                        } else if (EPI == EPI_MASK) {
                            // BF16 > 0: sign bit clear and not +0 (the bits of a positive value)
                            const uint32_t m = mw[j / 2];
                            const uint32_t m0 = m & 0xffffu, m1 = m >> 16;
                            x0 = (m0 != 0u && m0 < 0x8000u && m0 <= 0x7f80u) ? x0 : 0.0f;
                            x1 = (m1 != 0u && m1 < 0x8000u && m1 <= 0x7f80u) ? x1 : 0.0f;
                        }
                        pk[j / 2] = (uint32_t)f2bf(x0) | ((uint32_t)f2bf(x1) << 16);
                    }
                    if (nval == 32) {
                        uint4 *o4 = reinterpret_cast<uint4 *>(o);
#pragma unroll
                        for (int tt = 0; tt < 4; ++tt)
                            o4[tt] = make_uint4(pk[4 * tt], pk[4 * tt + 1], pk[4 * tt + 2], pk[4 * tt + 3]);
                    } else {
                        uint32_t *o2 = reinterpret_cast<uint32_t *>(o);
#pragma unroll
                        for (int tt = 0; tt < 16; ++tt)
                            if (tt < nval / 2) o2[tt] = pk[tt];
                    }
                }
            }
            // this warp's reads of the buffer are complete: the MMA warp may reuse it
            tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&tempty[ab]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, 2u * (uint32_t)p.ncols);
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

static PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

cudaError_t tensor_map(CUtensorMap *m, const void *ptr, int rank, const uint64_t *dims, const uint64_t *strides,
                       const uint32_t *box, int row_bytes) {
    if (!g_encode) {
        cudaDriverEntryPointQueryResult q;
        void *fn = nullptr;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
        if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !fn) return e != cudaSuccess ? e : cudaErrorNotSupported;
        g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    }
    // the inner box row must fill the swizzle span exactly: TMA would pad a
    // narrower row to the span and overrun the shared-memory stage
    if (box[0] * 2u != (uint32_t)row_bytes) return cudaErrorInvalidValue;
    cuuint64_t gd[5], gs[4];
    cuuint32_t bd[5], es[5];
    for (int i = 0; i < rank; ++i) {
        gd[i] = dims[i];
        bd[i] = box[i];
        es[i] = 1;
        if (i + 1 < rank) gs[i] = strides[i];
    }
    const CUtensorMapSwizzle swz = row_bytes == 128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_64B;
    CUresult r = g_encode(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, (cuuint32_t)rank, const_cast<void *>(ptr), gd, gs, bd,
                          es, CU_TENSOR_MAP_INTERLEAVE_NONE, swz, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                          CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

static int pow2_cols(int n) {
    int c = 32;
    while (c < n) c <<= 1;
    return c;
}

static uint32_t kb_round(size_t b) { return (uint32_t)((b + 1023) / 1024 * 1024); }

static size_t smem_bytes(const GemmParams &p, int gy) {
    return 1024 + (size_t)p.stages * (p.aStage + p.bStage) + p.bres + 8 * (2 * p.stages + 6) + 16 +
           4 * (size_t)gy * p.N;
}

// stages of the given size in ~200 KB (the copy engine keeps few operations in
// flight per SM, so more than a handful of stages buys nothing)
static int pick_stages(uint32_t aStage, uint32_t bStage) {
    int s = (int)((200 * 1024) / (aStage + bStage));
    return s > 8 ? 8 : (s < 2 ? 2 : s);
}

// Persistent launch: min(tiles, SMs) CTAs (one per SM: ~200 KB of stages)
// walk the gx x gy x gz tiles.
template <int MODE, int EPI>
static cudaError_t launch(const CUtensorMap &A, const CUtensorMap &B, GemmParams p, dim3 tiles, cudaStream_t st) {
    const size_t smem = smem_bytes(p, (int)tiles.y);
    if (smem > 227 * 1024) return cudaErrorInvalidValue;
    cudaError_t e = cudaFuncSetAttribute(umma_kernel<MODE, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    const int sms = device_sms();
    p.gx = (int)tiles.x;
    p.gy = (int)tiles.y;
    p.gz = (int)tiles.z;
    p.ntiles = (long long)tiles.x * tiles.y * tiles.z;
    if (p.ntiles == 0) return cudaSuccess;
    const unsigned grid = (unsigned)(p.ntiles < sms ? p.ntiles : sms);
    umma_kernel<MODE, EPI><<<grid, 192, smem, st>>>(A, B, p);
    return cudaGetLastError();
}

cudaError_t gemm_bf16(const uint16_t *A, const uint16_t *B, float *C, int M, int N, int K, int *err,
                      unsigned long long limit_ns, cudaStream_t st) {
    if (M % 128 || N % 16 || N > 256 || N < 16 || K % 64) return cudaErrorInvalidValue;
    GemmParams p = {};
    p.M = M;
    p.N = N;
    p.ncols = pow2_cols(N);
    p.kbytes = 128;
    p.nk = K / 64;
    p.aStage = 128u * 128u;
    p.bStage = kb_round((size_t)N * 128);
    p.stages = pick_stages(p.aStage, p.bStage);
    p.bytesA = 128u * 128u;
    p.bytesB = (uint32_t)N * 128u;
    p.out = C;
    p.ldo = N;
    p.err = err;
    p.limit_ns = limit_ns;
    CUtensorMap ta, tb;
    const uint64_t da[2] = {(uint64_t)K, (uint64_t)M}, sa[1] = {(uint64_t)K * 2};
    const uint32_t ba[2] = {64, 128};
    const uint64_t db[2] = {(uint64_t)K, (uint64_t)N}, sb[1] = {(uint64_t)K * 2};
    const uint32_t bb[2] = {64, (uint32_t)N};
    cudaError_t e;
    if ((e = tensor_map(&ta, A, 2, da, sa, ba, 128)) != cudaSuccess) return e;
    if ((e = tensor_map(&tb, B, 2, db, sb, bb, 128)) != cudaSuccess) return e;
    return launch<MODE_GEMM, EPI_F32>(ta, tb, p, dim3(M / 128, 1, 1), st);
}

// wp[(cc*9 + tap)*Cout + o][j] = w[o][tap*Cin + 64*cc + j] (0 past Cin): the
// weights of the row-strip form, 64-channel chunks, taps and output channels
// as rows of 128 bytes.
__global__ void pack_weights_kernel(const uint16_t *__restrict__ w, uint16_t *__restrict__ wp, int Cin, int Cout,
                                    int cchunks) {
    const long long n = (long long)cchunks * 9 * Cout * 64;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(i & 63);
        const long long r = i >> 6;
        const int o = (int)(r % Cout);
        const int t = (int)(r / Cout);          // cc*9 + tap
        const int cc = t / 9, tap = t - cc * 9;
        const int c = 64 * cc + j;
        wp[i] = c < Cin ? w[(long long)o * 9 * Cin + tap * Cin + c] : (uint16_t)0;
    }
}

// Image rows of 128k pixels: a tile is 128 pixels of one row, and per input
// row ky and 64-channel chunk ONE strip of 130 pixels (halo of one on each
// side) is loaded, with the three taps' weights as one more box; the taps kx
// are views of the strip shifted by kx rows.  Compared with a box per tap
// this issues a third of the copy operations and moves a third of the input.
static cudaError_t conv3x3_halo(const ConvArgs &c, int epi, int ntile, int *err, unsigned long long limit_ns,
                                cudaStream_t st) {
    GemmParams p = {};
    p.N = ntile;
    p.ncols = pow2_cols(ntile);
    p.kbytes = 128;
    p.cchunks = (c.Cin + 63) / 64;
    p.nk = 3 * p.cchunks;
    p.aStage = kb_round(130u * 128u);
    // weights resident when one n tile covers Cout and they leave room for 4 strips
    const size_t bfull_bytes = (size_t)p.cchunks * 9 * ntile * 128;
    const bool resident = ntile == c.Cout && bfull_bytes + 4 * (size_t)p.aStage <= 200u * 1024u;
    if (resident) {
        p.bres = (uint32_t)bfull_bytes;
        p.bStage = 0;
        const int s = (int)((200u * 1024u - bfull_bytes) / p.aStage);
        p.stages = s > 8 ? 8 : s;
    } else {
        p.bStage = kb_round(3u * (size_t)ntile * 128u);
        p.stages = pick_stages(p.aStage, p.bStage);
    }
    p.H = c.H;
    p.W = c.W;
    p.Cin = c.Cin;
    p.bw = 128;
    p.bh = 1;
    p.bytesA = 130u * 128u;
    p.bytesB = resident ? 0u : 3u * (uint32_t)ntile * 128u;
    p.out = c.y;
    p.ldo = c.ldy;
    p.coff = c.yoff;
    p.bias = c.bias;
    p.mask = c.mask;
    p.ldm = c.ldm;
    p.moff = c.moff;
    p.err = err;
    p.limit_ns = limit_ns;
    // packed weights in stream-ordered scratch
    const long long npk = (long long)p.cchunks * 9 * c.Cout * 64;
    uint16_t *wp = nullptr;
    cudaError_t e = cudaMallocAsync(reinterpret_cast<void **>(&wp), (size_t)npk * 2, st);
    if (e != cudaSuccess) return e;
    pack_weights_kernel<<<(unsigned)((npk + 255) / 256 < 1024 ? (npk + 255) / 256 : 1024), 256, 0, st>>>(
        c.w, wp, c.Cin, c.Cout, p.cchunks);
    if ((e = cudaGetLastError()) != cudaSuccess) {
        cudaFreeAsync(wp, st);
        return e;
    }
    CUtensorMap ta, tb;
    const uint64_t da[4] = {(uint64_t)c.Cin, (uint64_t)c.W, (uint64_t)c.H, (uint64_t)c.B};
    const uint64_t sa[3] = {(uint64_t)c.ldx * 2, (uint64_t)c.ldx * 2 * c.W, (uint64_t)c.ldx * 2 * c.W * c.H};
    const uint32_t ba[4] = {64, 130, 1, 1};
    const uint64_t db[3] = {64, (uint64_t)c.Cout, (uint64_t)p.cchunks * 9};
    const uint64_t sb[2] = {128, (uint64_t)c.Cout * 128};
    const uint32_t bbx[3] = {64, (uint32_t)ntile, resident ? (uint32_t)(p.cchunks * 9) : 3u};
    const dim3 grid((unsigned)((long long)c.B * c.H * c.W / 128), (unsigned)(c.Cout / ntile), 1);
    if ((e = tensor_map(&ta, c.x + c.xoff, 4, da, sa, ba, 128)) == cudaSuccess &&
        (e = tensor_map(&tb, wp, 3, db, sb, bbx, 128)) == cudaSuccess) {
        switch (epi) {
            case EPI_BIAS_RELU: e = launch<MODE_HALO, EPI_BIAS_RELU>(ta, tb, p, grid, st); break;
            case EPI_BIAS: e = launch<MODE_HALO, EPI_BIAS>(ta, tb, p, grid, st); break;
            case EPI_MASK: e = launch<MODE_HALO, EPI_MASK>(ta, tb, p, grid, st); break;
            default: e = cudaErrorInvalidValue;
        }
    }
    const cudaError_t e2 = cudaFreeAsync(wp, st);
    return e != cudaSuccess ? e : e2;
}

cudaError_t conv3x3(const ConvArgs &c, int epi, int *err, unsigned long long limit_ns, cudaStream_t st) {
    if (c.Cin % 32 || c.Cout % 16 || (c.ldx % 8) || (c.xoff % 8) || (c.ldy % 8) || (c.yoff % 8))
        return cudaErrorInvalidValue;
    if (epi == EPI_MASK && (!c.mask || (c.ldm % 8) || (c.moff % 8))) return cudaErrorInvalidValue;
    // N tiles of at most 256 output channels (TMEM columns / UMMA N)
    const int ntile = c.Cout <= 256 ? c.Cout : (c.Cout % 192 == 0 ? 192 : (c.Cout % 128 == 0 ? 128 : 0));
    if (ntile == 0) return cudaErrorInvalidValue;
    // the row-strip form when a tile is one image row and two stages fit
    if (c.W % 128 == 0 && kb_round(130u * 128u) + kb_round(3u * (size_t)ntile * 128u) <= 100u * 1024u)
        return conv3x3_halo(c, epi, ntile, err, limit_ns, st);
    const int bw = c.W >= 128 ? 128 : c.W;
    const int bh = 128 / bw;
    if (128 % bw || c.W % bw || c.H % bh) return cudaErrorInvalidValue;
    // K chunks of 64 channels (128-byte rows, 128-byte swizzle) where Cin allows,
    // else 32 (64-byte rows): TMA moves long rows at a higher rate
    const int cw = c.Cin % 64 == 0 ? 64 : 32;
    const int kb = 2 * cw;
    GemmParams p = {};
    p.N = ntile;
    p.ncols = pow2_cols(ntile);
    p.kbytes = kb;
    p.cchunks = c.Cin / cw;
    p.nk = 9 * p.cchunks;
    p.aStage = 128u * (uint32_t)kb;
    p.bStage = kb_round((size_t)ntile * kb);
    p.stages = pick_stages(p.aStage, p.bStage);
    p.H = c.H;
    p.W = c.W;
    p.Cin = c.Cin;
    p.bw = bw;
    p.bh = bh;
    p.bytesA = 128u * (uint32_t)kb;
    p.bytesB = (uint32_t)ntile * (uint32_t)kb;
    p.out = c.y;
    p.ldo = c.ldy;
    p.coff = c.yoff;
    p.bias = c.bias;
    p.mask = c.mask;
    p.ldm = c.ldm;
    p.moff = c.moff;
    p.err = err;
    p.limit_ns = limit_ns;
    CUtensorMap ta, tb;
    const uint64_t da[4] = {(uint64_t)c.Cin, (uint64_t)c.W, (uint64_t)c.H, (uint64_t)c.B};
    const uint64_t sa[3] = {(uint64_t)c.ldx * 2, (uint64_t)c.ldx * 2 * c.W, (uint64_t)c.ldx * 2 * c.W * c.H};
    const uint32_t ba[4] = {(uint32_t)cw, (uint32_t)bw, (uint32_t)bh, 1};
    const uint64_t db[2] = {(uint64_t)9 * c.Cin, (uint64_t)c.Cout}, sb[1] = {(uint64_t)9 * c.Cin * 2};
    const uint32_t bbx[2] = {(uint32_t)cw, (uint32_t)ntile};
    cudaError_t e;
    if ((e = tensor_map(&ta, c.x + c.xoff, 4, da, sa, ba, kb)) != cudaSuccess) return e;
    if ((e = tensor_map(&tb, c.w, 2, db, sb, bbx, kb)) != cudaSuccess) return e;
    const dim3 grid((unsigned)((long long)c.B * c.H * c.W / 128), (unsigned)(c.Cout / ntile), 1);
    switch (epi) {
        case EPI_BIAS_RELU: return launch<MODE_CONV, EPI_BIAS_RELU>(ta, tb, p, grid, st);
        case EPI_BIAS: return launch<MODE_CONV, EPI_BIAS>(ta, tb, p, grid, st);
        case EPI_MASK: return launch<MODE_CONV, EPI_MASK>(ta, tb, p, grid, st);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t conv3x3_wgrad(const WgradArgs &w, int *err, unsigned long long limit_ns, cudaStream_t st) {
    if (w.Cin % 16 || w.Cout % 16) return cudaErrorInvalidValue;
    // A K chunk is one run of pixels of one image row whose bytes are exactly
    // the swizzle span (TMA pads a narrower box row to the span in shared
    // memory): 64 pixels / 128-byte swizzle, or 32 pixels / 64-byte swizzle.
    const int bwk = w.W >= 64 ? 64 : 32;
    const int bhk = 1;
    if (w.W % bwk) return cudaErrorInvalidValue;
    const int kbytes = bwk * 2;
    const int ntile = w.Cin <= 256 ? w.Cin : (w.Cin % 192 == 0 ? 192 : 128);
    if (w.Cin % ntile) return cudaErrorInvalidValue;
    // a stage holds a super-chunk of kw x kh pixel chunks (4 where the image
    // allows): one TMA box per operand per stage
    const int nwb = w.W / bwk;
    const int arows = w.Cout < 128 ? w.Cout : 128;
    int kw = 1, kh = 1;
    for (int nsub = 4; nsub >= 1; nsub /= 2) {      // the largest that leaves room for two stages
        const int tw = nwb >= nsub ? nsub : nwb;
        const int th = nsub / tw;
        if (nwb % tw || w.H % th) continue;
        const size_t stage = kb_round(((size_t)(nsub - 1) * arows + 128) * kbytes) +
                             kb_round((size_t)nsub * ntile * kbytes);
        if (2 * stage <= 200u * 1024u) {
            kw = tw;
            kh = th;
            break;
        }
    }
    GemmParams p = {};
    p.N = ntile;
    p.ncols = pow2_cols(ntile);
    p.kbytes = kbytes;
    p.kw = kw;
    p.kh = kh;
    p.arows = arows;
    // the M = 128 MMA of the last sub-chunk reads 128 rows from its start
    p.aStage = kb_round(((size_t)(kw * kh - 1) * arows + 128) * kbytes);
    p.bStage = kb_round((size_t)kw * kh * ntile * kbytes);
    p.stages = pick_stages(p.aStage, p.bStage);
    p.Cin = w.Cin;
    p.bwk = bwk;
    p.bhk = bhk;
    p.nb_w = nwb / kw;
    p.nb_h = w.H / kh;
    p.Bn = w.B;
    p.ksplit = w.ksplit;
    p.mvalid = w.Cout;
    p.bytesA = (uint32_t)(kw * kh * arows * kbytes);
    p.bytesB = (uint32_t)(kw * kh * ntile * kbytes);
    p.out = w.dw;
    p.ldo = 9LL * w.Cin;
    p.err = err;
    p.limit_ns = limit_ns;
    CUtensorMap ta, tb;
    const uint64_t nwbu = (uint64_t)nwb;
    const uint64_t da[5] = {(uint64_t)bwk, (uint64_t)w.Cout, nwbu, (uint64_t)w.H, (uint64_t)w.B};
    const uint64_t sa[4] = {(uint64_t)bwk * 2, (uint64_t)w.Cout * bwk * 2, nwbu * w.Cout * bwk * 2,
                            (uint64_t)w.H * nwbu * w.Cout * bwk * 2};
    const uint32_t ba[5] = {(uint32_t)bwk, (uint32_t)arows, (uint32_t)kw, (uint32_t)kh, 1};
    const uint64_t db[5] = {(uint64_t)bwk, (uint64_t)w.Cin, nwbu, (uint64_t)w.H, (uint64_t)3 * w.B};
    const uint64_t sb[4] = {(uint64_t)bwk * 2, (uint64_t)w.Cin * bwk * 2, nwbu * w.Cin * bwk * 2,
                            (uint64_t)w.H * nwbu * w.Cin * bwk * 2};
    const uint32_t bbx[5] = {(uint32_t)bwk, (uint32_t)ntile, (uint32_t)kw, (uint32_t)kh, 1};
    cudaError_t e;
    if ((e = tensor_map(&ta, w.dyT, 5, da, sa, ba, kbytes)) != cudaSuccess) return e;
    if ((e = tensor_map(&tb, w.xT3, 5, db, sb, bbx, kbytes)) != cudaSuccess) return e;
    const dim3 grid((unsigned)((w.Cout + 127) / 128), (unsigned)(w.Cin / ntile), (unsigned)(9 * w.ksplit));
    return launch<MODE_WGRAD, EPI_ATOMIC>(ta, tb, p, grid, st);
}

}  // namespace unet
}  // namespace synk

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
//               input channels in chunks of 32; the A box of a tap is the
//               tile's 128 pixels shifted by the tap, read from a 4-D map
//               (C, W, H, batch) whose out-of-bounds zeros are the padding.
//               The backward-data pass is the same convolution of the output
//               gradient with the tap-flipped, transposed weights.
//   MODE_WGRAD  weight gradient: K = pixels (64 per chunk) of channel-major
//               copies, A = dY^T (output channels), B = X^T shifted by the tap
//               (three copies pre-shifted along W; the H shift is the TMA
//               coordinate), split over K across CTAs with FP32 atomics.
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

template <int MODE, int EPI>
__global__ void __launch_bounds__(192, 1) umma_kernel(const __grid_constant__ CUtensorMap tmA,
                                                      const __grid_constant__ CUtensorMap tmB, const GemmParams p) {
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    uint8_t *smem = smem_raw + (((raw + 1023u) & ~1023u) - raw);
    const uint32_t aBytes = 128u * (uint32_t)p.kbytes;
    const uint32_t bBytes = (((uint32_t)p.N * (uint32_t)p.kbytes + 1023u) / 1024u) * 1024u;
    const uint32_t stageBytes = aBytes + bBytes;
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + (size_t)p.stages * stageBytes);
    uint64_t *empty = full + p.stages;
    uint64_t *accum = empty + p.stages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accum + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (warp == 0) {
        tmem_alloc(tmem_slot, (uint32_t)p.ncols);
        tmem_relinquish();
    }
    if (warp == 1 && lane == 0) {
        for (int s = 0; s < p.stages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        fence_mbar_init();
    }
    if (warp == 0 && lane == 0) {
        tma_prefetch_desc(&tmA);
        tma_prefetch_desc(&tmB);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    // ---- this CTA's tile and K range ----
    int m0 = 0, n0 = blockIdx.y * p.N, kbeg = 0, nk = p.nk;
    int b = 0, h0 = 0, w0 = 0, ky = 0, kx = 0;
    if (MODE == MODE_GEMM) {
        m0 = blockIdx.x * 128;
    } else if (MODE == MODE_CONV) {
        const int tiles_w = p.W / p.bw, tpi = tiles_w * (p.H / p.bh);
        const int mt = blockIdx.x;
        b = mt / tpi;
        const int r = mt - b * tpi;
        h0 = (r / tiles_w) * p.bh;
        w0 = (r - (r / tiles_w) * tiles_w) * p.bw;
    } else {   // MODE_WGRAD
        m0 = blockIdx.x * 128;
        const int tap = blockIdx.z / p.ksplit, ks = blockIdx.z - tap * p.ksplit;
        ky = tap / 3;
        kx = tap - ky * 3;
        const long long nbk = (long long)p.Bn * p.nb_h * p.nb_w;
        kbeg = (int)(nbk * ks / p.ksplit);
        nk = (int)(nbk * (ks + 1) / p.ksplit) - kbeg;
    }

    if (warp == 0) {
        if (lane == 0) {
            // ---- TMA producer ----
            int issued = 0;
            for (int kc = 0; kc < nk; ++kc) {
                const int s = kc % p.stages;
                const uint32_t ph = (uint32_t)(kc / p.stages) & 1u;
                if (kc >= p.stages && !mbar_wait(&empty[s], ph ^ 1u, p.err, p.limit_ns)) break;
                uint8_t *As = smem + (size_t)s * stageBytes;
                uint8_t *Bs = As + aBytes;
                mbar_arrive_expect_tx(&full[s], p.bytesA + p.bytesB);
                if (MODE == MODE_GEMM) {
                    const int ke = p.kbytes / 2;
                    tma_load_2d(As, &tmA, &full[s], kc * ke, m0);
                    tma_load_2d(Bs, &tmB, &full[s], kc * ke, n0);
                } else if (MODE == MODE_CONV) {
                    const int tap = kc / p.cchunks, cc = kc - tap * p.cchunks;
                    const int tky = tap / 3, tkx = tap - tky * 3;
                    tma_load_4d(As, &tmA, &full[s], cc * 32, w0 + tkx - 1, h0 + tky - 1, b);
                    tma_load_2d(Bs, &tmB, &full[s], tap * p.Cin + cc * 32, n0);
                } else {
                    const int pb = kbeg + kc;
                    const int per_img = p.nb_h * p.nb_w;
                    const int bb = pb / per_img;
                    const int r = pb - bb * per_img;
                    const int hb = r / p.nb_w, wb = r - (r / p.nb_w) * p.nb_w;
                    tma_load_4d(As, &tmA, &full[s], wb * p.bwk, hb * p.bhk, bb, m0);
                    tma_load_4d(Bs, &tmB, &full[s], wb * p.bwk, hb * p.bhk + ky - 1, bb, kx * p.Cin + n0);
                }
                issued = kc + 1;
            }
            // no copy may still be landing when the CTA exits: wait for the last
            // use of every stage (immediate on the normal path)
            const int first = issued > p.stages ? issued - p.stages : 0;
            for (int kc = first; kc < issued; ++kc)
                mbar_wait(&full[kc % p.stages], (uint32_t)(kc / p.stages) & 1u, p.err, p.limit_ns);
        }
    } else if (warp == 1) {
        if (lane == 0) {
            // ---- MMA issuer ----
            const uint32_t idesc = idesc_bf16(128, p.N);
            const uint32_t kbytes = (uint32_t)p.kbytes;
            for (int kc = 0; kc < nk; ++kc) {
                const int s = kc % p.stages;
                const uint32_t ph = (uint32_t)(kc / p.stages) & 1u;
                if (!mbar_wait(&full[s], ph, p.err, p.limit_ns)) break;
                tc_fence_after();
                const uint32_t a0 = smem_u32(smem + (size_t)s * stageBytes);
                const uint32_t b0 = a0 + aBytes;
                for (uint32_t kk = 0; kk < kbytes / 32u; ++kk) {
                    mma_bf16(tmem, smem_desc(a0 + kk * 32u, kbytes), smem_desc(b0 + kk * 32u, kbytes), idesc,
                             (kc | (int)kk) != 0 ? 1u : 0u);
                }
                mma_commit(&empty[s]);
            }
            mma_commit(accum);     // also issued on an early exit: completes when issued MMAs have
        }
    } else {
        // ---- epilogue (warps 2..5) ----
        const int q = warp & 3;
        const int row = q * 32 + lane;
        const bool ok = mbar_wait(accum, 0u, p.err, p.limit_ns) && nk > 0;
        tc_fence_after();
        // tcgen05.ld is warp-collective: decide once per warp
        const bool good = __all_sync(0xffffffffu, ok && *(volatile int *)p.err == 0);
        // output position of this row
        long long pix = 0;
        bool rvalid = true;
        if (MODE == MODE_GEMM) {
            rvalid = m0 + row < p.M;
        } else if (MODE == MODE_CONV) {
            const int h = h0 + row / p.bw, w = w0 + (row - (row / p.bw) * p.bw);
            pix = ((long long)b * p.H + h) * p.W + w;
        } else {
            rvalid = m0 + row < p.mvalid;
        }
        for (int c0 = 0; c0 < p.N; c0 += 32) {
            float v[32];
            if (good) tmem_ld_32x32(tmem + ((uint32_t)(q * 32) << 16) + (uint32_t)c0, v);
            if (!good || !rvalid) continue;
            const int nbase = n0 + c0;
            const int nval = min(32, p.N - c0);
            if (EPI == EPI_F32) {
                float *o = reinterpret_cast<float *>(p.out) + (long long)(m0 + row) * p.ldo + nbase;
                for (int j = 0; j < nval; ++j) o[j] = v[j];
            } else if (EPI == EPI_ATOMIC) {
                const int tap = blockIdx.z / p.ksplit;
                float *o = reinterpret_cast<float *>(p.out) + (long long)(m0 + row) * p.ldo + tap * p.Cin + nbase;
                const int lim = min(nval, p.Cin - nbase);
                for (int j = 0; j < lim; ++j) atomicAdd(o + j, v[j]);
            } else {
                uint16_t *o = reinterpret_cast<uint16_t *>(p.out) + pix * p.ldo + p.coff + nbase;
                uint32_t pk[16];
#pragma unroll
                for (int j = 0; j < 32; j += 2) {
                    float x0 = v[j], x1 = v[j + 1];
                    if (EPI == EPI_BIAS_RELU || EPI == EPI_BIAS) {
                        x0 += p.bias[nbase + j];
                        x1 += p.bias[nbase + j + 1];
                        if (EPI == EPI_BIAS_RELU) {
                            x0 = fmaxf(x0, 0.0f);
                            x1 = fmaxf(x1, 0.0f);
                        }
                    } else if (EPI == EPI_MASK) {
                        const uint16_t *mk = p.mask + pix * p.ldm + p.moff + nbase + j;
                        x0 = bf2f(mk[0]) > 0.0f ? x0 : 0.0f;
                        x1 = bf2f(mk[1]) > 0.0f ? x1 : 0.0f;
                    }
                    pk[j / 2] = (uint32_t)f2bf(x0) | ((uint32_t)f2bf(x1) << 16);
                }
                if (nval == 32) {
                    uint4 *o4 = reinterpret_cast<uint4 *>(o);
#pragma unroll
                    for (int t = 0; t < 4; ++t) o4[t] = make_uint4(pk[4 * t], pk[4 * t + 1], pk[4 * t + 2], pk[4 * t + 3]);
                } else {
                    uint32_t *o2 = reinterpret_cast<uint32_t *>(o);
                    for (int t = 0; t < nval / 2; ++t) o2[t] = pk[t];
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tmem_dealloc(tmem, (uint32_t)p.ncols);
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

static size_t smem_bytes(const GemmParams &p) {
    const size_t a = 128u * p.kbytes, b = ((size_t)p.N * p.kbytes + 1023) / 1024 * 1024;
    return 1024 + (size_t)p.stages * (a + b) + 8 * (2 * p.stages + 1) + 16;
}

static int pick_stages(int N, int kbytes) {
    const size_t a = 128u * kbytes, b = ((size_t)N * kbytes + 1023) / 1024 * 1024;
    int s = (int)((200 * 1024) / (a + b));
    return s > 8 ? 8 : (s < 2 ? 2 : s);
}

template <int MODE, int EPI>
static cudaError_t launch(const CUtensorMap &A, const CUtensorMap &B, const GemmParams &p, dim3 grid,
                          cudaStream_t st) {
    const size_t smem = smem_bytes(p);
    cudaError_t e = cudaFuncSetAttribute(umma_kernel<MODE, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
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
    p.stages = pick_stages(N, 128);
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

cudaError_t conv3x3(const ConvArgs &c, int epi, int *err, unsigned long long limit_ns, cudaStream_t st) {
    if (c.Cin % 32 || c.Cout % 16 || (c.ldx % 8) || (c.xoff % 8) || (c.ldy % 8) || (c.yoff % 8))
        return cudaErrorInvalidValue;
    // N tiles of at most 256 output channels (TMEM columns / UMMA N)
    const int ntile = c.Cout <= 256 ? c.Cout : (c.Cout % 192 == 0 ? 192 : (c.Cout % 128 == 0 ? 128 : 0));
    if (ntile == 0) return cudaErrorInvalidValue;
    const int bw = c.W >= 128 ? 128 : c.W;
    const int bh = 128 / bw;
    if (128 % bw || c.W % bw || c.H % bh) return cudaErrorInvalidValue;
    GemmParams p = {};
    p.N = ntile;
    p.ncols = pow2_cols(ntile);
    p.kbytes = 64;
    p.cchunks = c.Cin / 32;
    p.nk = 9 * p.cchunks;
    p.stages = pick_stages(ntile, 64);
    p.H = c.H;
    p.W = c.W;
    p.Cin = c.Cin;
    p.bw = bw;
    p.bh = bh;
    p.bytesA = 128u * 64u;
    p.bytesB = (uint32_t)ntile * 64u;
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
    const uint32_t ba[4] = {32, (uint32_t)bw, (uint32_t)bh, 1};
    const uint64_t db[2] = {(uint64_t)9 * c.Cin, (uint64_t)c.Cout}, sb[1] = {(uint64_t)9 * c.Cin * 2};
    const uint32_t bbx[2] = {32, (uint32_t)ntile};
    cudaError_t e;
    if ((e = tensor_map(&ta, c.x + c.xoff, 4, da, sa, ba, 64)) != cudaSuccess) return e;
    if ((e = tensor_map(&tb, c.w, 2, db, sb, bbx, 64)) != cudaSuccess) return e;
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
    GemmParams p = {};
    p.N = ntile;
    p.ncols = pow2_cols(ntile);
    p.kbytes = kbytes;
    p.stages = pick_stages(ntile, kbytes);
    p.Cin = w.Cin;
    p.bwk = bwk;
    p.bhk = bhk;
    p.nb_w = w.W / bwk;
    p.nb_h = w.H / bhk;
    p.Bn = w.B;
    p.ksplit = w.ksplit;
    p.mvalid = w.Cout;
    const int arows = w.Cout < 128 ? w.Cout : 128;
    p.bytesA = (uint32_t)arows * (uint32_t)kbytes;
    p.bytesB = (uint32_t)ntile * (uint32_t)kbytes;
    p.out = w.dw;
    p.ldo = 9LL * w.Cin;
    p.err = err;
    p.limit_ns = limit_ns;
    CUtensorMap ta, tb;
    const uint64_t pix = (uint64_t)w.B * w.H * w.W;
    const uint64_t da[4] = {(uint64_t)w.W, (uint64_t)w.H, (uint64_t)w.B, (uint64_t)w.Cout};
    const uint64_t sa[3] = {(uint64_t)w.W * 2, (uint64_t)w.W * w.H * 2, pix * 2};
    const uint32_t ba[4] = {(uint32_t)bwk, (uint32_t)bhk, 1, (uint32_t)arows};
    const uint64_t db[4] = {(uint64_t)w.W, (uint64_t)w.H, (uint64_t)w.B, (uint64_t)3 * w.Cin};
    const uint32_t bbx[4] = {(uint32_t)bwk, (uint32_t)bhk, 1, (uint32_t)ntile};
    cudaError_t e;
    if ((e = tensor_map(&ta, w.dyT, 4, da, sa, ba, kbytes)) != cudaSuccess) return e;
    if ((e = tensor_map(&tb, w.xT3, 4, db, sa, bbx, kbytes)) != cudaSuccess) return e;
    const dim3 grid((unsigned)((w.Cout + 127) / 128), (unsigned)(w.Cin / ntile), (unsigned)(9 * w.ksplit));
    return launch<MODE_WGRAD, EPI_ATOMIC>(ta, tb, p, grid, st);
}

}  // namespace unet
}  // namespace synk

// CUDA-core kernels around the tcgen05 convolutions of the U-Net warm
// starter: the 1-channel input layer, 2x2 max pooling, 2x nearest
// upsampling into concatenation buffers, the 1x1 output head with the MSE
// loss, channel-major (transposed, W-shifted) copies for the weight gradient,
// bias gradients and the fused Adam update.  Activations are BF16 NHWC with a
// channel stride `ld` (so a tensor can be a channel slice of a wider buffer).
#include <cuda_bf16.h>

#include "unet_ops.cuh"

namespace synk {
namespace unet {

__device__ __forceinline__ float bf(uint16_t x) { return __bfloat162float(__ushort_as_bfloat16(x)); }
__device__ __forceinline__ uint16_t tobf(float x) { return __bfloat16_as_ushort(__float2bfloat16_rn(x)); }

// Eight BF16 channels travel as one 16-byte vector (channel strides and
// offsets are multiples of 8, checked on the host).
__device__ __forceinline__ void unpack8(const uint4 u, float (&f)[8]) {
    const uint32_t w[4] = {u.x, u.y, u.z, u.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
        f[2 * i] = __uint_as_float(w[i] << 16);
        f[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
    }
}
__device__ __forceinline__ uint4 pack8(const float (&f)[8]) {
    uint32_t w[4];
#pragma unroll
    for (int i = 0; i < 4; ++i) w[i] = (uint32_t)tobf(f[2 * i]) | ((uint32_t)tobf(f[2 * i + 1]) << 16);
    return make_uint4(w[0], w[1], w[2], w[3]);
}
__device__ __forceinline__ uint4 ld8(const uint16_t *p) { return *reinterpret_cast<const uint4 *>(p); }
__device__ __forceinline__ void st8(uint16_t *p, uint4 v) { *reinterpret_cast<uint4 *>(p) = v; }

// e[b,h,w,o] = relu(bias[o] + sum_tap x[b,h+dy,w+dx] * w[o][tap]), x FP32 1
// channel; one thread per pixel, all Cout (<= 64, multiple of 8) outputs.
__global__ void __launch_bounds__(256) first_conv_kernel(const float *__restrict__ x, const float *__restrict__ w,
                                                         const float *__restrict__ bias, uint16_t *__restrict__ y,
                                                         int B, int H, int W, int Cout, int ldy) {
    __shared__ float sw[64 * 9], sb[64];
    for (int i = threadIdx.x; i < Cout * 9; i += blockDim.x) sw[i] = w[i];
    for (int i = threadIdx.x; i < Cout; i += blockDim.x) sb[i] = bias[i];
    __syncthreads();
    const unsigned P = (unsigned)B * H * W;
    for (unsigned p = blockIdx.x * blockDim.x + threadIdx.x; p < P; p += gridDim.x * blockDim.x) {
        const unsigned w0 = p % W, t = p / W, h0 = t % H;
        float v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const int h = (int)h0 + k / 3 - 1, ww = (int)w0 + k % 3 - 1;
            v[k] = (h >= 0 && h < H && ww >= 0 && ww < W) ? __ldg(x + (long long)p + (k / 3 - 1) * W + (k % 3 - 1))
                                                          : 0.0f;
        }
        uint16_t *o = y + (long long)p * ldy;
        for (int c0 = 0; c0 < Cout; c0 += 8) {
            float r[8];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                float s = sb[c0 + j];
#pragma unroll
                for (int k = 0; k < 9; ++k) s = fmaf(v[k], sw[(c0 + j) * 9 + k], s);
                r[j] = fmaxf(s, 0.0f);
            }
            st8(o + c0, pack8(r));
        }
    }
}

// dw[o][tap] += sum_p dz[p][o] * x[p + tap]; db[o] += sum_p dz[p][o], Cout = 32.
// Thread (pixel, group of 8 channels); lanes with the same group reduce by
// shuffles, warps through shared memory, one atomic per (o, tap) per block.
__global__ void __launch_bounds__(256) first_conv_wgrad_kernel(const float *__restrict__ x,
                                                               const uint16_t *__restrict__ dz, int ldz,
                                                               float *__restrict__ dw, float *__restrict__ db, int B,
                                                               int H, int W) {
    const int grp = threadIdx.x & 3;                    // channels 8*grp .. +7
    const unsigned P = (unsigned)B * H * W;
    float acc[8][10];
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int k = 0; k < 10; ++k) acc[j][k] = 0.0f;
    const unsigned stride = gridDim.x * (blockDim.x >> 2);
    for (unsigned p = blockIdx.x * (blockDim.x >> 2) + (threadIdx.x >> 2); p < P; p += stride) {
        float g[8];
        unpack8(ld8(dz + (long long)p * ldz + 8 * grp), g);
        const unsigned w0 = p % W, t = p / W, h0 = t % H;
        float v[9];
#pragma unroll
        for (int k = 0; k < 9; ++k) {
            const int h = (int)h0 + k / 3 - 1, ww = (int)w0 + k % 3 - 1;
            v[k] = (h >= 0 && h < H && ww >= 0 && ww < W) ? __ldg(x + (long long)p + (k / 3 - 1) * W + (k % 3 - 1))
                                                          : 0.0f;
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
#pragma unroll
            for (int k = 0; k < 9; ++k) acc[j][k] = fmaf(g[j], v[k], acc[j][k]);
            acc[j][9] += g[j];
        }
    }
    __shared__ float red[8][4][80];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
        for (int k = 0; k < 10; ++k) {
            float a = acc[j][k];
            a += __shfl_xor_sync(0xffffffffu, a, 4);
            a += __shfl_xor_sync(0xffffffffu, a, 8);
            a += __shfl_xor_sync(0xffffffffu, a, 16);
            if (lane < 4) red[warp][lane][j * 10 + k] = a;
        }
    __syncthreads();
    for (int i = threadIdx.x; i < 320; i += blockDim.x) {
        const int gg = i / 80, jk = i - gg * 80;
        float s = 0.0f;
        for (int wi = 0; wi < (int)(blockDim.x >> 5); ++wi) s += red[wi][gg][jk];
        const int o = 8 * gg + jk / 10, k = jk % 10;
        atomicAdd(k < 9 ? dw + o * 9 + k : db + o, s);
    }
}

// out[b,h,w,c] = max of the 2x2 block of in (H, W of the input); thread =
// (output pixel, 8 channels).
__global__ void __launch_bounds__(256) maxpool_kernel(const uint16_t *__restrict__ in, int ldi, int ioff,
                                                      uint16_t *__restrict__ out, int ldo, int B, int H, int W, int C) {
    const unsigned Ho = H / 2, Wo = W / 2, G = C / 8;
    const unsigned n = (unsigned)B * Ho * Wo * G;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned g = i % G, q = i / G;
        const unsigned wo = q % Wo, t = q / Wo, ho = t % Ho, b = t / Ho;
        const long long r0 = ((long long)b * H + 2 * ho) * W + 2 * wo;
        const int c = ioff + 8 * (int)g;
        float a0[8], a1[8], a2[8], a3[8];
        unpack8(ld8(in + r0 * ldi + c), a0);
        unpack8(ld8(in + (r0 + 1) * ldi + c), a1);
        unpack8(ld8(in + (r0 + W) * ldi + c), a2);
        unpack8(ld8(in + (r0 + W + 1) * ldi + c), a3);
#pragma unroll
        for (int j = 0; j < 8; ++j) a0[j] = fmaxf(fmaxf(a0[j], a1[j]), fmaxf(a2[j], a3[j]));
        st8(out + (long long)q * ldo + 8 * g, pack8(a0));
    }
}

// dE[b,h,w,c] = dP[b,h/2,w/2,c] where (h,w) holds the block's max (first in
// scan order), plus the skip gradient dS[b,h,w,c] when given; thread =
// (pooled pixel, 8 channels), writing its 2x2 block.
__global__ void __launch_bounds__(256) maxpool_bwd_kernel(const uint16_t *__restrict__ e, int lde, int eoff,
                                                          const uint16_t *__restrict__ dp, int ldp,
                                                          const uint16_t *__restrict__ ds, int lds, int soff,
                                                          uint16_t *__restrict__ de, int ldd, int B, int H, int W,
                                                          int C) {
    const unsigned Ho = H / 2, Wo = W / 2, G = C / 8;
    const unsigned n = (unsigned)B * Ho * Wo * G;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned g = i % G, q = i / G;
        const unsigned wo = q % Wo, t = q / Wo, ho = t % Ho, b = t / Ho;
        const long long r0 = ((long long)b * H + 2 * ho) * W + 2 * wo;
        const long long rr[4] = {r0, r0 + 1, r0 + W, r0 + W + 1};
        float a[4][8], gp[8];
#pragma unroll
        for (int k = 0; k < 4; ++k) unpack8(ld8(e + rr[k] * lde + eoff + 8 * g), a[k]);
        unpack8(ld8(dp + (long long)q * ldp + 8 * g), gp);
        float o[4][8];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            int am = 0;
            float best = a[0][j];
#pragma unroll
            for (int k = 1; k < 4; ++k)
                if (a[k][j] > best) {
                    best = a[k][j];
                    am = k;
                }
#pragma unroll
            for (int k = 0; k < 4; ++k) o[k][j] = (k == am) ? gp[j] : 0.0f;
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            if (ds) {
                float sk[8];
                unpack8(ld8(ds + rr[k] * lds + soff + 8 * g), sk);
#pragma unroll
                for (int j = 0; j < 8; ++j) o[k][j] += sk[j];
            }
            st8(de + rr[k] * ldd + 8 * g, pack8(o[k]));
        }
    }
}

// out[b,h,w,ooff+c] = in[b,h/2,w/2,c] (output H, W); thread = (output pixel, 8 channels).
__global__ void __launch_bounds__(256) upsample_kernel(const uint16_t *__restrict__ in, int ldi,
                                                       uint16_t *__restrict__ out, int ldo, int ooff, int B, int H,
                                                       int W, int C) {
    const unsigned G = C / 8;
    const unsigned n = (unsigned)B * H * W * G;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned g = i % G, q = i / G;
        const unsigned w = q % W, t = q / W, h = t % H, b = t / H;
        const long long src = ((long long)b * (H / 2) + h / 2) * (W / 2) + w / 2;
        st8(out + (long long)q * ldo + ooff + 8 * g, ld8(in + src * ldi + 8 * g));
    }
}

// out[b,h,w,c] = sum of the 2x2 children in[b,2h+i,2w+j,ioff+c] (output H, W);
// thread = (output pixel, 8 channels).
__global__ void __launch_bounds__(256) upsample_bwd_kernel(const uint16_t *__restrict__ in, int ldi, int ioff,
                                                           uint16_t *__restrict__ out, int ldo, int B, int H, int W,
                                                           int C) {
    const unsigned G = C / 8;
    const unsigned n = (unsigned)B * H * W * G;
    const int W2 = 2 * W;
    for (unsigned i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const unsigned g = i % G, q = i / G;
        const unsigned w = q % W, t = q / W, h = t % H, b = t / H;
        const long long r0 = ((long long)b * 2 * H + 2 * h) * W2 + 2 * w;
        const int c = ioff + 8 * (int)g;
        float s0[8], s1[8], s2[8], s3[8];
        unpack8(ld8(in + r0 * ldi + c), s0);
        unpack8(ld8(in + (r0 + 1) * ldi + c), s1);
        unpack8(ld8(in + (r0 + W2) * ldi + c), s2);
        unpack8(ld8(in + (r0 + W2 + 1) * ldi + c), s3);
#pragma unroll
        for (int j = 0; j < 8; ++j) s0[j] = s0[j] + s1[j] + s2[j] + s3[j];
        st8(out + (long long)q * ldo + 8 * g, pack8(s0));
    }
}

// Output head and loss: y = x0 + bh + sum_c wh[c] * d[p][c] (C <= 64, multiple
// of 8); with a target, g = 2 (y - t) / P and loss += (y - t)^2 / P (FP64).
__global__ void __launch_bounds__(256) head_kernel(const float *__restrict__ x0, const uint16_t *__restrict__ d,
                                                   int ldd, const float *__restrict__ wh, const float *__restrict__ bh,
                                                   float *__restrict__ y, const float *__restrict__ target,
                                                   float *__restrict__ g, double *__restrict__ loss, long long P,
                                                   int C) {
    __shared__ float sw[64];
    for (int i = threadIdx.x; i < C; i += blockDim.x) sw[i] = wh[i];
    __syncthreads();
    double l = 0.0;
    const float b0 = bh[0];
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        float s = x0[p] + b0;
        for (int c0 = 0; c0 < C; c0 += 8) {
            float dv[8];
            unpack8(ld8(d + p * ldd + c0), dv);
#pragma unroll
            for (int j = 0; j < 8; ++j) s = fmaf(sw[c0 + j], dv[j], s);
        }
        if (y) y[p] = s;
        if (target) {
            const float r = s - target[p];
            g[p] = 2.0f * r / (float)P;
            l += (double)r * r;
        }
    }
    if (!target) return;
#pragma unroll
    for (int o = 16; o; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    __shared__ double sh[8];
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh[i];
        atomicAdd(loss, t / (double)P);
    }
}

// Head backward (C = 32): dz[p][c] = g[p] * wh[c] * (d[p][c] > 0);
// dwh[c] += sum_p g d; dbh += sum g.
__global__ void __launch_bounds__(256) head_bwd_kernel(const float *__restrict__ g, const uint16_t *__restrict__ d,
                                                       int ldd, const float *__restrict__ wh,
                                                       uint16_t *__restrict__ dz, int ldz, float *__restrict__ dwh,
                                                       float *__restrict__ dbh, long long P, int C) {
    __shared__ float sw[32];
    __shared__ float red[8][33];
    for (int i = threadIdx.x; i < 32; i += blockDim.x) sw[i] = i < C ? wh[i] : 0.0f;
    __syncthreads();
    float acc[33];
#pragma unroll
    for (int c = 0; c < 33; ++c) acc[c] = 0.0f;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        const float gp = g[p];
#pragma unroll
        for (int c0 = 0; c0 < 32; c0 += 8) {
            float dv[8], o[8];
            unpack8(ld8(d + p * ldd + c0), dv);
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                o[j] = dv[j] > 0.0f ? gp * sw[c0 + j] : 0.0f;
                acc[c0 + j] = fmaf(gp, dv[j], acc[c0 + j]);
            }
            st8(dz + p * ldz + c0, pack8(o));
        }
        acc[32] += gp;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
#pragma unroll
    for (int c = 0; c < 33; ++c) {
        float a = acc[c];
#pragma unroll
        for (int o = 16; o; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        if (lane == 0) red[warp][c] = a;
    }
    __syncthreads();
    if (threadIdx.x < 33 && (threadIdx.x < (unsigned)C || threadIdx.x == 32)) {
        float s = 0.0f;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i][threadIdx.x];
        atomicAdd(threadIdx.x < 32 ? dwh + threadIdx.x : dbh, s);
    }
}

// Blocked copies for the weight gradient: pixel chunks of cw pixels of one
// image row (cw = 64 when W >= 64, else 32), each chunk stored as [C][cw].
// shifted = 0: out[q][c][j] = in[q*cw + j][c] (one copy); shifted = 1: three
// copies, copy k at k*P*C, holding in[p + k - 1][c] when pixel p+k-1 is in
// p's image row (w+k-1 in [0, W)), else 0.  A block handles 128 pixels (plus
// one halo pixel on each side) x 64 channels: 16-byte loads into a
// channel-major shared tile, then 16-byte stores of 8 consecutive pixels of
// one channel, so each warp writes whole 128-byte lines.
__global__ void __launch_bounds__(256) to_cmajor_kernel(const uint16_t *__restrict__ in, int ldi, int ioff,
                                                        uint16_t *__restrict__ out, int C, long long P, int W,
                                                        int shifted) {
    __shared__ uint16_t tile[64][130];   // [channel][pixel p0-1 .. p0+128]; 65-word rows
    const long long p0 = (long long)blockIdx.x * 128;
    const int c0 = blockIdx.y * 64;
    const int cn = min(64, C - c0);      // multiple of 8
    const int G = cn / 8;
    const int cw = W >= 64 ? 64 : 32;
    for (int i = threadIdx.x; i < 130 * G; i += blockDim.x) {
        const int r = i / G, h = i - r * G;
        const long long p = p0 - 1 + r;
        uint4 v = make_uint4(0u, 0u, 0u, 0u);
        if (p >= 0 && p < P) v = ld8(in + p * ldi + ioff + c0 + 8 * h);
        const uint32_t wv[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int k = 0; k < 8; ++k) tile[8 * h + k][r] = (uint16_t)((k & 1) ? (wv[k >> 1] >> 16) : (wv[k >> 1] & 0xffffu));
    }
    __syncthreads();
    const int ncopies = shifted ? 3 : 1;
    // thread = (channel c, group g of 8 pixels); groups fastest
    for (int i = threadIdx.x; i < 16 * cn; i += blockDim.x) {
        const int g = i & 15, c = i >> 4;
        const long long p = p0 + 8 * g;
        if (p >= P) continue;            // P is a multiple of 8: a group is wholly in or out
        const int w0 = (int)(p % W);     // the group lies in one image row (W multiple of 8)
        const long long q = p / cw;
        const int j = (int)(p - q * cw);
        for (int k = 0; k < ncopies; ++k) {
            const int dsh = shifted ? k - 1 : 0;
            uint32_t wv[4];
#pragma unroll
            for (int e = 0; e < 8; e += 2) {
                const bool in0 = w0 + e + dsh >= 0 && w0 + e + dsh < W;
                const bool in1 = w0 + e + 1 + dsh >= 0 && w0 + e + 1 + dsh < W;
                const uint32_t v0 = in0 ? tile[c][8 * g + e + 1 + dsh] : 0u;
                const uint32_t v1 = in1 ? tile[c][8 * g + e + 2 + dsh] : 0u;
                wv[e >> 1] = v0 | (v1 << 16);
            }
            uint16_t *o = out + (long long)k * P * C + (q * C + c0 + c) * cw + j;
            *reinterpret_cast<uint4 *>(o) = make_uint4(wv[0], wv[1], wv[2], wv[3]);
        }
    }
}

// db[c] += sum_p dz[p][c].  Thread = (channel group g of 8, pixel lane): a block
// covers G = C/8 groups x 256/G pixel lanes, 16-byte loads; lanes of one
// group are summed in shared memory, one atomic per channel per block.
__global__ void __launch_bounds__(256) bias_grad_kernel(const uint16_t *__restrict__ dz, int ldz,
                                                        float *__restrict__ db, long long P, int C) {
    const int G = C / 8;
    const int lanes = blockDim.x / G;                  // pixel lanes per block
    const int g = threadIdx.x % G, pl = threadIdx.x / G;
    float acc[8] = {0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f, 0.0f};
    if (pl < lanes)
        for (long long p = (long long)blockIdx.x * lanes + pl; p < P; p += (long long)gridDim.x * lanes) {
            float v[8];
            unpack8(ld8(dz + p * ldz + 8 * g), v);
#pragma unroll
            for (int j = 0; j < 8; ++j) acc[j] += v[j];
        }
    __shared__ float sh[256][9];
#pragma unroll
    for (int j = 0; j < 8; ++j) sh[threadIdx.x][j] = pl < lanes ? acc[j] : 0.0f;
    __syncthreads();
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        const int gg = c / 8, j = c % 8;
        float t = 0.0f;
        for (int l = 0; l < lanes; ++l) t += sh[l * G + gg][j];
        atomicAdd(db + c, t);
    }
}

// Fused Adam (bias-corrected): per parameter, g -> m, v -> w; the gradient is
// zeroed for the next step.  For 3x3 weights [Cout][9][Cin] the BF16 copy and
// the tap-flipped transposed BF16 copy [Cin][9][Cout] of the backward-data
// convolution are written in the same pass.
__global__ void adam_kernel(float *__restrict__ w, float *__restrict__ g, float *__restrict__ m,
                            float *__restrict__ v, long long n, float lr, float b1, float b2, float eps, float c1,
                            float c2, uint16_t *__restrict__ wbf, uint16_t *__restrict__ wtbf, int Cout, int Cin) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float gi = g[i];
        const float mi = b1 * m[i] + (1.0f - b1) * gi;
        const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        const float wi = w[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps);
        w[i] = wi;
        g[i] = 0.0f;
        if (wbf) {
            wbf[i] = tobf(wi);
            if (wtbf) {
                const int ci = (int)(i % Cin), tap = (int)((i / Cin) % 9), co = (int)(i / (9LL * Cin));
                wtbf[((long long)ci * 9 + (8 - tap)) * Cout + co] = tobf(wi);
            }
        }
    }
}

// BF16 copies of 3x3 weights (forward and flipped-transposed) without an update.
__global__ void weights_bf16_kernel(const float *__restrict__ w, long long n, uint16_t *__restrict__ wbf,
                                    uint16_t *__restrict__ wtbf, int Cout, int Cin) {
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const float wi = w[i];
        wbf[i] = tobf(wi);
        if (wtbf) {
            const int ci = (int)(i % Cin), tap = (int)((i / Cin) % 9), co = (int)(i / (9LL * Cin));
            wtbf[((long long)ci * 9 + (8 - tap)) * Cout + co] = tobf(wi);
        }
    }
}

static unsigned grid_for(long long n, int threads = 256) {
    long long g = (n + threads - 1) / threads;
    if (g > 152LL * 16) g = 152LL * 16;
    return (unsigned)(g < 1 ? 1 : g);
}

static bool v8(int a) { return (a & 7) == 0; }

cudaError_t first_conv(const float *x, const float *w, const float *b, uint16_t *y, int B, int H, int W, int Cout,
                       int ldy, cudaStream_t st) {
    if (!v8(Cout) || Cout > 64 || !v8(ldy) || (long long)B * H * W >= (1LL << 31)) return cudaErrorInvalidValue;
    first_conv_kernel<<<grid_for((long long)B * H * W), 256, 0, st>>>(x, w, b, y, B, H, W, Cout, ldy);
    return cudaGetLastError();
}
cudaError_t first_conv_wgrad(const float *x, const uint16_t *dz, int ldz, float *dw, float *db, int B, int H, int W,
                             int Cout, cudaStream_t st) {
    if (Cout != 32 || !v8(ldz) || (long long)B * H * W >= (1LL << 31)) return cudaErrorInvalidValue;
    first_conv_wgrad_kernel<<<152 * 2, 256, 0, st>>>(x, dz, ldz, dw, db, B, H, W);
    return cudaGetLastError();
}
cudaError_t maxpool(const uint16_t *in, int ldi, int ioff, uint16_t *out, int ldo, int B, int H, int W, int C,
                    cudaStream_t st) {
    const long long n = (long long)B * (H / 2) * (W / 2) * (C / 8);
    if (!v8(C) || !v8(ldi) || !v8(ioff) || !v8(ldo) || n >= (1LL << 31)) return cudaErrorInvalidValue;
    maxpool_kernel<<<grid_for(n), 256, 0, st>>>(in, ldi, ioff, out, ldo, B, H, W, C);
    return cudaGetLastError();
}
cudaError_t maxpool_bwd(const uint16_t *e, int lde, int eoff, const uint16_t *dp, int ldp, const uint16_t *ds,
                        int lds, int soff, uint16_t *de, int ldd, int B, int H, int W, int C, cudaStream_t st) {
    const long long n = (long long)B * (H / 2) * (W / 2) * (C / 8);
    if (!v8(C) || !v8(lde) || !v8(eoff) || !v8(ldp) || !v8(lds) || !v8(soff) || !v8(ldd) || n >= (1LL << 31))
        return cudaErrorInvalidValue;
    maxpool_bwd_kernel<<<grid_for(n), 256, 0, st>>>(e, lde, eoff, dp, ldp, ds, lds, soff, de, ldd, B, H, W, C);
    return cudaGetLastError();
}
cudaError_t upsample(const uint16_t *in, int ldi, uint16_t *out, int ldo, int ooff, int B, int H, int W, int C,
                     cudaStream_t st) {
    const long long n = (long long)B * H * W * (C / 8);
    if (!v8(C) || !v8(ldi) || !v8(ldo) || !v8(ooff) || n >= (1LL << 31)) return cudaErrorInvalidValue;
    upsample_kernel<<<grid_for(n), 256, 0, st>>>(in, ldi, out, ldo, ooff, B, H, W, C);
    return cudaGetLastError();
}
cudaError_t upsample_bwd(const uint16_t *in, int ldi, int ioff, uint16_t *out, int ldo, int B, int H, int W, int C,
                         cudaStream_t st) {
    const long long n = (long long)B * H * W * (C / 8);
    if (!v8(C) || !v8(ldi) || !v8(ioff) || !v8(ldo) || n >= (1LL << 31)) return cudaErrorInvalidValue;
    upsample_bwd_kernel<<<grid_for(n), 256, 0, st>>>(in, ldi, ioff, out, ldo, B, H, W, C);
    return cudaGetLastError();
}
cudaError_t head(const float *x0, const uint16_t *d, int ldd, const float *wh, const float *bh, float *y,
                 const float *target, float *g, double *loss, long long P, int C, cudaStream_t st) {
    if (!v8(C) || C > 64 || !v8(ldd)) return cudaErrorInvalidValue;
    head_kernel<<<grid_for(P), 256, 0, st>>>(x0, d, ldd, wh, bh, y, target, g, loss, P, C);
    return cudaGetLastError();
}
cudaError_t head_bwd(const float *g, const uint16_t *d, int ldd, const float *wh, uint16_t *dz, int ldz, float *dwh,
                     float *dbh, long long P, int C, cudaStream_t st) {
    if (C != 32 || !v8(ldd) || !v8(ldz)) return cudaErrorInvalidValue;
    head_bwd_kernel<<<152 * 4, 256, 0, st>>>(g, d, ldd, wh, dz, ldz, dwh, dbh, P, C);
    return cudaGetLastError();
}
cudaError_t to_cmajor(const uint16_t *in, int ldi, int ioff, uint16_t *out, int C, long long P, int W, int shifted,
                      cudaStream_t st) {
    if (!v8(C) || !v8(ldi) || !v8(ioff) || W < 32 || W % (W >= 64 ? 64 : 32) || P % W)
        return cudaErrorInvalidValue;
    dim3 grid((unsigned)((P + 127) / 128), (unsigned)((C + 63) / 64));
    to_cmajor_kernel<<<grid, 256, 0, st>>>(in, ldi, ioff, out, C, P, W, shifted);
    return cudaGetLastError();
}
cudaError_t bias_grad(const uint16_t *dz, int ldz, float *db, long long P, int C, cudaStream_t st) {
    if (!v8(C) || C > 2048 || !v8(ldz)) return cudaErrorInvalidValue;
    bias_grad_kernel<<<152 * 2, 256, 0, st>>>(dz, ldz, db, P, C);
    return cudaGetLastError();
}
cudaError_t adam(float *w, float *g, float *m, float *v, long long n, float lr, float b1, float b2, float eps, int step,
                 uint16_t *wbf, uint16_t *wtbf, int Cout, int Cin, cudaStream_t st) {
    const float c1 = 1.0f - powf(b1, (float)step), c2 = 1.0f - powf(b2, (float)step);
    adam_kernel<<<grid_for(n), 256, 0, st>>>(w, g, m, v, n, lr, b1, b2, eps, c1, c2, wbf, wtbf, Cout, Cin);
    return cudaGetLastError();
}
cudaError_t weights_bf16(const float *w, long long n, uint16_t *wbf, uint16_t *wtbf, int Cout, int Cin,
                         cudaStream_t st) {
    weights_bf16_kernel<<<grid_for(n), 256, 0, st>>>(w, n, wbf, wtbf, Cout, Cin);
    return cudaGetLastError();
}

}  // namespace unet
}  // namespace synk

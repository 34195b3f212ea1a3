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

// e[b,h,w,o] = relu(bias[o] + sum_tap x[b,h+dy,w+dx] * w[o][tap]), x FP32 1 channel.
__global__ void first_conv_kernel(const float *__restrict__ x, const float *__restrict__ w,
                                  const float *__restrict__ bias, uint16_t *__restrict__ y, int B, int H, int W,
                                  int Cout, int ldy) {
    const long long P = (long long)B * H * W;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        const int w0 = (int)(p % W), h0 = (int)((p / W) % H);
        const long long b = p / ((long long)W * H);
        float v[9];
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            const int h = h0 + t / 3 - 1, ww = w0 + t % 3 - 1;
            v[t] = (h >= 0 && h < H && ww >= 0 && ww < W) ? x[(b * H + h) * W + ww] : 0.0f;
        }
        uint16_t *o = y + p * ldy;
        for (int c = 0; c < Cout; ++c) {
            float s = bias[c];
#pragma unroll
            for (int t = 0; t < 9; ++t) s = fmaf(v[t], w[c * 9 + t], s);
            o[c] = tobf(fmaxf(s, 0.0f));
        }
    }
}

// dw[o][tap] += sum_p dz[p][o] * x[p + tap]; db[o] += sum_p dz[p][o].  One block
// per (o, slice of pixels); shared-memory reduction, one atomic per block.
__global__ void first_conv_wgrad_kernel(const float *__restrict__ x, const uint16_t *__restrict__ dz, int ldz,
                                        float *__restrict__ dw, float *__restrict__ db, int B, int H, int W) {
    const int o = blockIdx.y;
    const long long P = (long long)B * H * W;
    float acc[10] = {0};
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        const float g = bf(dz[p * ldz + o]);
        if (g == 0.0f) continue;
        const int w0 = (int)(p % W), h0 = (int)((p / W) % H);
        const long long b = p / ((long long)W * H);
#pragma unroll
        for (int t = 0; t < 9; ++t) {
            const int h = h0 + t / 3 - 1, ww = w0 + t % 3 - 1;
            if (h >= 0 && h < H && ww >= 0 && ww < W) acc[t] = fmaf(g, x[(b * H + h) * W + ww], acc[t]);
        }
        acc[9] += g;
    }
    __shared__ float sh[10][256];
#pragma unroll
    for (int t = 0; t < 10; ++t) sh[t][threadIdx.x] = acc[t];
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s)
            for (int t = 0; t < 10; ++t) sh[t][threadIdx.x] += sh[t][threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x < 9) atomicAdd(dw + o * 9 + threadIdx.x, sh[threadIdx.x][0]);
    if (threadIdx.x == 9) atomicAdd(db + o, sh[9][0]);
}

// out[b,h,w,c] = max of the 2x2 block of in (H, W of the input).
__global__ void maxpool_kernel(const uint16_t *__restrict__ in, int ldi, int ioff, uint16_t *__restrict__ out, int ldo,
                               int B, int H, int W, int C) {
    const int Ho = H / 2, Wo = W / 2;
    const long long n = (long long)B * Ho * Wo * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long q = i / C;
        const int wo = (int)(q % Wo), ho = (int)((q / Wo) % Ho);
        const long long b = q / ((long long)Wo * Ho);
        const long long r0 = (b * H + 2 * ho) * W + 2 * wo;
        const float a0 = bf(in[r0 * ldi + ioff + c]), a1 = bf(in[(r0 + 1) * ldi + ioff + c]);
        const float a2 = bf(in[(r0 + W) * ldi + ioff + c]), a3 = bf(in[(r0 + W + 1) * ldi + ioff + c]);
        out[q * ldo + c] = tobf(fmaxf(fmaxf(a0, a1), fmaxf(a2, a3)));
    }
}

// dE[b,h,w,c] (+)= dP[b,h/2,w/2,c] where (h,w) holds the block's max (first in
// scan order), plus the skip gradient dS[b,h,w,c] when given.
__global__ void maxpool_bwd_kernel(const uint16_t *__restrict__ e, int lde, int eoff, const uint16_t *__restrict__ dp,
                                   int ldp, const uint16_t *__restrict__ ds, int lds, int soff,
                                   uint16_t *__restrict__ de, int ldd, int B, int H, int W, int C) {
    const long long n = (long long)B * H * W * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long q = i / C;
        const int w = (int)(q % W), h = (int)((q / W) % H);
        const long long b = q / ((long long)W * H);
        const int hb = h & ~1, wb = w & ~1;
        const long long r0 = (b * H + hb) * W + wb;
        const float a[4] = {bf(e[r0 * lde + eoff + c]), bf(e[(r0 + 1) * lde + eoff + c]),
                            bf(e[(r0 + W) * lde + eoff + c]), bf(e[(r0 + W + 1) * lde + eoff + c])};
        int am = 0;
        for (int t = 1; t < 4; ++t)
            if (a[t] > a[am]) am = t;
        const int me = (h - hb) * 2 + (w - wb);
        float g = 0.0f;
        if (me == am) g = bf(dp[((b * (H / 2) + h / 2) * (W / 2) + w / 2) * ldp + c]);
        if (ds) g += bf(ds[q * lds + soff + c]);
        de[q * ldd + c] = tobf(g);
    }
}

// out[b,h,w,ooff+c] = in[b,h/2,w/2,c] (output H, W).
__global__ void upsample_kernel(const uint16_t *__restrict__ in, int ldi, uint16_t *__restrict__ out, int ldo,
                                int ooff, int B, int H, int W, int C) {
    const long long n = (long long)B * H * W * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long q = i / C;
        const int w = (int)(q % W), h = (int)((q / W) % H);
        const long long b = q / ((long long)W * H);
        out[q * ldo + ooff + c] = in[((b * (H / 2) + h / 2) * (W / 2) + w / 2) * ldi + c];
    }
}

// out[b,h,w,c] = sum of the 2x2 children in[b,2h+i,2w+j,ioff+c] (output H, W).
__global__ void upsample_bwd_kernel(const uint16_t *__restrict__ in, int ldi, int ioff, uint16_t *__restrict__ out,
                                    int ldo, int B, int H, int W, int C) {
    const long long n = (long long)B * H * W * C;
    const int W2 = 2 * W;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long q = i / C;
        const int w = (int)(q % W), h = (int)((q / W) % H);
        const long long b = q / ((long long)W * H);
        const long long r0 = (b * 2 * H + 2 * h) * W2 + 2 * w;
        const float s = bf(in[r0 * ldi + ioff + c]) + bf(in[(r0 + 1) * ldi + ioff + c]) +
                        bf(in[(r0 + W2) * ldi + ioff + c]) + bf(in[(r0 + W2 + 1) * ldi + ioff + c]);
        out[q * ldo + c] = tobf(s);
    }
}

// Output head and loss: y = x0 + bh + sum_c wh[c] * d[p][c]; with a target,
// g = 2 (y - t) / P and loss += (y - t)^2 / P (FP64).
__global__ void head_kernel(const float *__restrict__ x0, const uint16_t *__restrict__ d, int ldd,
                            const float *__restrict__ wh, const float *__restrict__ bh, float *__restrict__ y,
                            const float *__restrict__ target, float *__restrict__ g, double *__restrict__ loss,
                            long long P, int C) {
    double l = 0.0;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        float s = x0[p] + bh[0];
        for (int c = 0; c < C; ++c) s = fmaf(wh[c], bf(d[p * ldd + c]), s);
        if (y) y[p] = s;
        if (target) {
            const float r = s - target[p];
            g[p] = 2.0f * r / (float)P;
            l += (double)r * r;
        }
    }
    if (!target) return;
    __shared__ double sh[256];
    sh[threadIdx.x] = l;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) atomicAdd(loss, sh[0] / (double)P);
}

// Head backward: dz[p][c] = g[p] * wh[c] * (d[p][c] > 0); dwh[c] += sum_p g d; dbh += sum g.
__global__ void head_bwd_kernel(const float *__restrict__ g, const uint16_t *__restrict__ d, int ldd,
                                const float *__restrict__ wh, uint16_t *__restrict__ dz, int ldz,
                                float *__restrict__ dwh, float *__restrict__ dbh, long long P, int C) {
    float acc[33];
    for (int c = 0; c <= C; ++c) acc[c] = 0.0f;
    for (long long p = (long long)blockIdx.x * blockDim.x + threadIdx.x; p < P; p += (long long)gridDim.x * blockDim.x) {
        const float gp = g[p];
        for (int c = 0; c < C; ++c) {
            const float dv = bf(d[p * ldd + c]);
            dz[p * ldz + c] = tobf(dv > 0.0f ? gp * wh[c] : 0.0f);
            acc[c] = fmaf(gp, dv, acc[c]);
        }
        acc[C] += gp;
    }
    __shared__ float sh[256];
    for (int c = 0; c <= C; ++c) {
        sh[threadIdx.x] = acc[c];
        __syncthreads();
        for (int s = blockDim.x / 2; s > 0; s >>= 1) {
            if ((int)threadIdx.x < s) sh[threadIdx.x] += sh[threadIdx.x + s];
            __syncthreads();
        }
        if (threadIdx.x == 0) atomicAdd(c < C ? dwh + c : dbh, sh[0]);
        __syncthreads();
    }
}

// Channel-major copies for the weight gradient.  mode 0: out[c][p] = in[p][c]
// (one copy); mode 1: three copies out[k][c][b][h][w] = in[b][h][w+k-1][c]
// (zero outside the image).  32 x 32 (pixel, channel) tiles through shared memory.
__global__ void to_cmajor_kernel(const uint16_t *__restrict__ in, int ldi, int ioff, uint16_t *__restrict__ out,
                                 int C, long long P, int W, int shifted) {
    __shared__ uint16_t tile[32][34];
    const long long p0 = (long long)blockIdx.x * 32;
    const int c0 = blockIdx.y * 32;
    for (int i = threadIdx.y; i < 32; i += 8) {
        const long long p = p0 + i;
        const int c = c0 + threadIdx.x;
        tile[i][threadIdx.x] = (p < P && c < C) ? in[p * ldi + ioff + c] : (uint16_t)0;
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += 8) {
        const int c = c0 + i;
        const long long p = p0 + threadIdx.x;
        if (c >= C || p >= P) continue;
        const uint16_t v = tile[threadIdx.x][i];
        if (!shifted) {
            out[(long long)c * P + p] = v;
        } else {
            // value at pixel p lands at p+1 in copy 0 (x[w-1]), p in copy 1, p-1 in copy 2
            const int w = (int)(p % W);
            out[(long long)(C + c) * P + p] = v;
            if (w + 1 < W) out[(long long)c * P + p + 1] = v;
            if (w >= 1) out[(long long)(2 * C + c) * P + p - 1] = v;
        }
    }
}

// Borders of the shifted copies: copy 0 at w = 0 and copy 2 at w = W-1 are zero.
__global__ void shift_border_kernel(uint16_t *__restrict__ out, int C, long long P, int W) {
    const long long rows = P / W;
    const long long n = rows * C;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % C);
        const long long r = i / C;
        out[(long long)c * P + r * W] = 0;
        out[(long long)(2 * C + c) * P + r * W + W - 1] = 0;
    }
}

// db[c] += sum_p dz[p][c]
__global__ void bias_grad_kernel(const uint16_t *__restrict__ dz, int ldz, float *__restrict__ db, long long P, int C) {
    const int c = blockIdx.y * 32 + (threadIdx.x & 31);
    float acc = 0.0f;
    if (c < C)
        for (long long p = (long long)blockIdx.x * (blockDim.x / 32) + threadIdx.x / 32; p < P;
             p += (long long)gridDim.x * (blockDim.x / 32))
            acc += bf(dz[p * ldz + c]);
    __shared__ float sh[8][33];
    sh[threadIdx.x / 32][threadIdx.x & 31] = acc;
    __syncthreads();
    if (threadIdx.x < 32) {
        float s = 0.0f;
        for (int i = 0; i < (int)blockDim.x / 32; ++i) s += sh[i][threadIdx.x];
        if (c < C) atomicAdd(db + c, s);
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

cudaError_t first_conv(const float *x, const float *w, const float *b, uint16_t *y, int B, int H, int W, int Cout,
                       int ldy, cudaStream_t st) {
    first_conv_kernel<<<grid_for((long long)B * H * W), 256, 0, st>>>(x, w, b, y, B, H, W, Cout, ldy);
    return cudaGetLastError();
}
cudaError_t first_conv_wgrad(const float *x, const uint16_t *dz, int ldz, float *dw, float *db, int B, int H, int W,
                             int Cout, cudaStream_t st) {
    dim3 grid(64, Cout);
    first_conv_wgrad_kernel<<<grid, 256, 0, st>>>(x, dz, ldz, dw, db, B, H, W);
    return cudaGetLastError();
}
cudaError_t maxpool(const uint16_t *in, int ldi, int ioff, uint16_t *out, int ldo, int B, int H, int W, int C,
                    cudaStream_t st) {
    maxpool_kernel<<<grid_for((long long)B * H * W * C / 4), 256, 0, st>>>(in, ldi, ioff, out, ldo, B, H, W, C);
    return cudaGetLastError();
}
cudaError_t maxpool_bwd(const uint16_t *e, int lde, int eoff, const uint16_t *dp, int ldp, const uint16_t *ds,
                        int lds, int soff, uint16_t *de, int ldd, int B, int H, int W, int C, cudaStream_t st) {
    maxpool_bwd_kernel<<<grid_for((long long)B * H * W * C), 256, 0, st>>>(e, lde, eoff, dp, ldp, ds, lds, soff, de,
                                                                          ldd, B, H, W, C);
    return cudaGetLastError();
}
cudaError_t upsample(const uint16_t *in, int ldi, uint16_t *out, int ldo, int ooff, int B, int H, int W, int C,
                     cudaStream_t st) {
    upsample_kernel<<<grid_for((long long)B * H * W * C), 256, 0, st>>>(in, ldi, out, ldo, ooff, B, H, W, C);
    return cudaGetLastError();
}
cudaError_t upsample_bwd(const uint16_t *in, int ldi, int ioff, uint16_t *out, int ldo, int B, int H, int W, int C,
                         cudaStream_t st) {
    upsample_bwd_kernel<<<grid_for((long long)B * H * W * C), 256, 0, st>>>(in, ldi, ioff, out, ldo, B, H, W, C);
    return cudaGetLastError();
}
cudaError_t head(const float *x0, const uint16_t *d, int ldd, const float *wh, const float *bh, float *y,
                 const float *target, float *g, double *loss, long long P, int C, cudaStream_t st) {
    head_kernel<<<grid_for(P), 256, 0, st>>>(x0, d, ldd, wh, bh, y, target, g, loss, P, C);
    return cudaGetLastError();
}
cudaError_t head_bwd(const float *g, const uint16_t *d, int ldd, const float *wh, uint16_t *dz, int ldz, float *dwh,
                     float *dbh, long long P, int C, cudaStream_t st) {
    head_bwd_kernel<<<grid_for(P), 256, 0, st>>>(g, d, ldd, wh, dz, ldz, dwh, dbh, P, C);
    return cudaGetLastError();
}
cudaError_t to_cmajor(const uint16_t *in, int ldi, int ioff, uint16_t *out, int C, long long P, int W, int shifted,
                      cudaStream_t st) {
    dim3 grid((unsigned)((P + 31) / 32), (unsigned)((C + 31) / 32));
    to_cmajor_kernel<<<grid, dim3(32, 8), 0, st>>>(in, ldi, ioff, out, C, P, W, shifted);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess || !shifted) return e;
    shift_border_kernel<<<grid_for(P / W * C), 256, 0, st>>>(out, C, P, W);
    return cudaGetLastError();
}
cudaError_t bias_grad(const uint16_t *dz, int ldz, float *db, long long P, int C, cudaStream_t st) {
    dim3 grid(256, (unsigned)((C + 31) / 32));
    bias_grad_kernel<<<grid, 256, 0, st>>>(dz, ldz, db, P, C);
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

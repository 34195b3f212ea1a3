// tcgen05 GEMM engine of the U-Net (umma_gemm.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace synk {
namespace unet {

enum { MODE_GEMM = 0, MODE_CONV = 1, MODE_WGRAD = 2, MODE_HALO = 3 };
enum { EPI_F32 = 0, EPI_BIAS_RELU = 1, EPI_MASK = 2, EPI_ATOMIC = 3, EPI_BIAS = 4 };

struct GemmParams {
    int M, N, ncols, nk, kbytes, stages;
    int gx, gy, gz;       // tile grid (x fastest); set by the launcher
    long long ntiles;
    uint32_t bytesA, bytesB;
    uint32_t aStage, bStage;   // bytes of the A and B parts of a stage (1 KB multiples)
    uint32_t bres;             // MODE_HALO: bytes of the B operand held resident (0: streamed per chunk)
    // MODE_CONV / MODE_HALO
    int H, W, Cin, bw, bh, cchunks;
    // MODE_WGRAD: K super-chunks of kw x kh pixel chunks (bwk pixels each) per stage
    int bwk, bhk, nb_w, nb_h, Bn, ksplit, mvalid, kw, kh, arows;
    // epilogue
    void *out;
    long long ldo;
    int coff;
    const float *bias;
    const uint16_t *mask;
    long long ldm;
    int moff;
    int *err;
    unsigned long long limit_ns;
};

// 3x3 convolution, pad 1, NHWC BF16 (channel slices of wider buffers allowed):
// y[b,h,w, yoff + o] = epi( sum_{tap,i} x[b, h+dy, w+dx, xoff + i] * w[o][tap*Cin + i] )
struct ConvArgs {
    const uint16_t *x;   // [B][H][W][ldx]
    int ldx, xoff, Cin;
    int B, H, W;
    const uint16_t *w;   // [Cout][9*Cin], tap = ky*3 + kx (dy = ky-1, dx = kx-1)
    const float *bias;   // [Cout] (EPI_BIAS*, else unused)
    uint16_t *y;         // [B][H][W][ldy]
    int ldy, yoff, Cout;
    const uint16_t *mask;   // EPI_MASK: y *= (mask[b,h,w, moff + o] > 0)
    long long ldm;
    int moff;
};

// weight gradient dw[o][tap*Cin + i] += sum_p dy[p][o] * x[p + tap offset][i]
struct WgradArgs {
    const uint16_t *dyT;   // [Cout][B][H][W] (channel-major output gradient)
    const uint16_t *xT3;   // [3][Cin][B][H][W]: copy kx holds x shifted by dx = kx-1 along W (zero outside)
    float *dw;             // [Cout][9*Cin], accumulated
    int Cin, Cout, B, H, W, ksplit;
};

cudaError_t gemm_bf16(const uint16_t *A, const uint16_t *B, float *C, int M, int N, int K, int *err,
                      unsigned long long limit_ns, cudaStream_t st);
cudaError_t conv3x3(const ConvArgs &c, int epi, int *err, unsigned long long limit_ns, cudaStream_t st);
cudaError_t conv3x3_wgrad(const WgradArgs &w, int *err, unsigned long long limit_ns, cudaStream_t st);

}  // namespace unet
}  // namespace synk

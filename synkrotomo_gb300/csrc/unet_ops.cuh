// CUDA-core kernels of the U-Net (unet_ops.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace synk {
namespace unet {

cudaError_t first_conv(const float *x, const float *w, const float *b, uint16_t *y, int B, int H, int W, int Cout,
                       int ldy, cudaStream_t st);
cudaError_t first_conv_wgrad(const float *x, const uint16_t *dz, int ldz, float *dw, float *db, int B, int H, int W,
                             int Cout, cudaStream_t st);
cudaError_t maxpool(const uint16_t *in, int ldi, int ioff, uint16_t *out, int ldo, int B, int H, int W, int C,
                    cudaStream_t st);
cudaError_t maxpool_bwd(const uint16_t *e, int lde, int eoff, const uint16_t *dp, int ldp, const uint16_t *ds,
                        int lds, int soff, uint16_t *de, int ldd, int B, int H, int W, int C, cudaStream_t st);
cudaError_t upsample(const uint16_t *in, int ldi, uint16_t *out, int ldo, int ooff, int B, int H, int W, int C,
                     cudaStream_t st);
cudaError_t upsample_bwd(const uint16_t *in, int ldi, int ioff, uint16_t *out, int ldo, int B, int H, int W, int C,
                         cudaStream_t st);
cudaError_t head(const float *x0, const uint16_t *d, int ldd, const float *wh, const float *bh, float *y,
                 const float *target, float *g, double *loss, long long P, int C, cudaStream_t st);
cudaError_t head_bwd(const float *g, const uint16_t *d, int ldd, const float *wh, uint16_t *dz, int ldz, float *dwh,
                     float *dbh, long long P, int C, cudaStream_t st);
cudaError_t to_cmajor(const uint16_t *in, int ldi, int ioff, uint16_t *out, int C, long long P, int W, int shifted,
                      cudaStream_t st);
cudaError_t bias_grad(const uint16_t *dz, int ldz, float *db, long long P, int C, cudaStream_t st);
cudaError_t adam(float *w, float *g, float *m, float *v, long long n, float lr, float b1, float b2, float eps, int step,
                 uint16_t *wbf, uint16_t *wtbf, int Cout, int Cin, cudaStream_t st);
cudaError_t weights_bf16(const float *w, long long n, uint16_t *wbf, uint16_t *wtbf, int Cout, int Cin,
                         cudaStream_t st);

}  // namespace unet
}  // namespace synk

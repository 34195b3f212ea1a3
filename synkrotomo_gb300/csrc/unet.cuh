// U-Net warm starter object (unet.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace synk {
namespace unet {

struct Net;

cudaError_t net_create(Net **out, int maxB, int N, unsigned long long seed, cudaStream_t st);
void net_free(Net *n);
long long net_nparams(const Net *n);
float *net_params(Net *n);   // device, FP32 [nparams]: per layer w [cout][9*cin] then b [cout]; head w [32], b
float *net_grads(Net *n);    // device, FP32 [nparams], same layout
float *net_adam_m(Net *n);   // device, FP32 [nparams]: Adam first moments
float *net_adam_v(Net *n);   // device, FP32 [nparams]: Adam second moments
int *net_adam_step(Net *n);  // host: Adam steps taken (bias correction)
double *net_loss(Net *n);    // device, the last forward's MSE
cudaError_t net_refresh_weights(Net *n, cudaStream_t st);
// y (optional) [B][N][N] = net(x); with target, the MSE goes to net_loss and
// the head gradient is prepared for net_backward.
cudaError_t net_forward(Net *n, int B, const float *x, float *y, const float *target, int *err,
                        unsigned long long lim, cudaStream_t st);
cudaError_t net_backward(Net *n, int B, int *err, unsigned long long lim, cudaStream_t st);
cudaError_t net_adam(Net *n, float lr, cudaStream_t st);

}  // namespace unet
}  // namespace synk

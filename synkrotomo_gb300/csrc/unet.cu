// U-Net warm starter (no counterpart in the reference): maps the normalised
// backprojection C*A^T*R*b of a sinogram to a start image for SIRT.
//
// Network (4 levels, 32 base channels, 3x3 convolutions with padding 1, ReLU,
// BF16 activations NHWC, FP32 accumulation and FP32 master weights):
//   level 1 (N):    conv 1->32 (CUDA cores), conv 32->32     -> e1
//   level 2 (N/2):  maxpool, conv 32->64, conv 64->64       -> e2
//   level 3 (N/4):  maxpool, conv 64->128, conv 128->128    -> e3
//   level 4 (N/8):  maxpool, conv 128->256, conv 256->256   -> e4
//   decoder:        upsample x2, concat skip, conv C->C/... (384->128, 128->128;
//                   192->64, 64->64; 96->32, 32->32)
//   head:           y = x + b + sum_c w[c] d1[c] (1x1 convolution, residual)
// Encoder outputs are written straight into the channel slices of the
// decoder's concatenation buffers (no copies).  All 3x3 convolutions after
// the first run on the tcgen05 engine (umma_gemm.cu): forward with fused
// bias+ReLU, backward-data as the convolution of the output gradient with the
// tap-flipped transposed weights with the ReLU mask fused, backward-weights
// over pixels.  Adam is one fused kernel per parameter tensor that also
// refreshes the BF16 weight copies.
#include <math.h>

#include <random>
#include <vector>

#include "synk_internal.cuh"
#include "umma_gemm.cuh"
#include "unet_ops.cuh"
#include "unet.cuh"

namespace synk {
namespace unet {

static const int kCin[14] = {1, 32, 32, 64, 64, 128, 128, 256, 384, 128, 192, 64, 96, 32};
static const int kCout[14] = {32, 32, 64, 64, 128, 128, 256, 256, 128, 128, 64, 64, 32, 32};
static const int kLevel[14] = {0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0};   // resolution N >> level

struct Layer {
    int cin, cout;
    long long woff, boff, nw;   // offsets into the flat parameter arrays
    uint16_t *wbf = nullptr;    // [cout][9*cin]
    uint16_t *wtbf = nullptr;   // [cin][9*cout], taps flipped
};

struct Net {
    int maxB = 0, N = 0, step = 0;
    long long nparams = 0, whoff = 0, bhoff = 0;
    Layer L[14];
    float *params = nullptr, *grads = nullptr, *m = nullptr, *v = nullptr;
    // activations (BF16 NHWC); level l has side N >> l
    uint16_t *e1a, *cat1, *p1, *e2a, *cat2, *p2, *e3a, *cat3, *p3, *e4a, *e4, *d3a, *d3, *d2a, *d2, *d1a, *d1;
    uint16_t *gA[4], *gB[4], *gcat1, *gcat2, *gcat3, *dzT, *xT3;
    float *x0, *tgt, *g;
    double *loss;
    std::vector<void *> allocs;

    template <class T>
    cudaError_t alloc(T **p, size_t n) {
        void *q = nullptr;
        cudaError_t e = cudaMalloc(&q, n * sizeof(T) + 256);
        if (e != cudaSuccess) return e;
        allocs.push_back(q);
        *p = static_cast<T *>(q);
        return cudaSuccess;
    }
    ~Net() {
        for (void *q : allocs) cudaFree(q);
    }
};

#define NET_TRY(call)                           \
    do {                                        \
        cudaError_t e_ = (call);                \
        if (e_ != cudaSuccess) return e_;       \
    } while (0)

cudaError_t net_create(Net **out, int maxB, int N, unsigned long long seed, cudaStream_t st) {
    if (N < 256 || N % 256 || maxB < 1) return cudaErrorInvalidValue;
    Net *n = new Net();
    n->maxB = maxB;
    n->N = N;
    long long off = 0;
    for (int l = 0; l < 14; ++l) {
        Layer &L = n->L[l];
        L.cin = kCin[l];
        L.cout = kCout[l];
        L.nw = 9LL * L.cin * L.cout;
        L.woff = off;
        off += L.nw;
        L.boff = off;
        off += L.cout;
    }
    n->whoff = off;
    off += 32;
    n->bhoff = off;
    off += 1;
    n->nparams = off;
    cudaError_t e;
#define A(ptr, cnt)                                           \
    if ((e = n->alloc(&(ptr), (size_t)(cnt))) != cudaSuccess) { \
        delete n;                                             \
        return e;                                             \
    }
    A(n->params, off);
    A(n->grads, off);
    A(n->m, off);
    A(n->v, off);
    for (int l = 1; l < 14; ++l) {
        A(n->L[l].wbf, n->L[l].nw);
        A(n->L[l].wtbf, n->L[l].nw);
    }
    const size_t P0 = (size_t)maxB * N * N;
    const size_t P1 = P0 / 4, P2 = P0 / 16, P3 = P0 / 64;
    A(n->e1a, P0 * 32);
    A(n->cat1, P0 * 96);
    A(n->p1, P1 * 32);
    A(n->e2a, P1 * 64);
    A(n->cat2, P1 * 192);
    A(n->p2, P2 * 64);
    A(n->e3a, P2 * 128);
    A(n->cat3, P2 * 384);
    A(n->p3, P3 * 128);
    A(n->e4a, P3 * 256);
    A(n->e4, P3 * 256);
    A(n->d3a, P2 * 128);
    A(n->d3, P2 * 128);
    A(n->d2a, P1 * 64);
    A(n->d2, P1 * 64);
    A(n->d1a, P0 * 32);
    A(n->d1, P0 * 32);
    const size_t Pl[4] = {P0, P1, P2, P3};
    const int Cl[4] = {32, 64, 128, 256};
    for (int l = 0; l < 4; ++l) {
        A(n->gA[l], Pl[l] * Cl[l]);
        A(n->gB[l], Pl[l] * Cl[l]);
    }
    A(n->gcat1, P0 * 96);
    A(n->gcat2, P1 * 192);
    A(n->gcat3, P2 * 384);
    // channel-major scratch of the weight gradient: largest C*P of any layer
    size_t dz_max = 0, x_max = 0;
    for (int l = 1; l < 14; ++l) {
        const size_t P = Pl[kLevel[l]];
        dz_max = dz_max > P * kCout[l] ? dz_max : P * kCout[l];
        x_max = x_max > 3 * P * kCin[l] ? x_max : 3 * P * kCin[l];
    }
    A(n->dzT, dz_max);
    A(n->xT3, x_max);
    A(n->x0, P0);
    A(n->tgt, P0);
    A(n->g, P0);
    A(n->loss, 1);
#undef A
    // He-normal initialisation (seeded), zero biases, small head
    std::vector<float> h((size_t)off, 0.0f);
    std::mt19937_64 rng(seed);
    for (int l = 0; l < 14; ++l) {
        std::normal_distribution<float> nd(0.0f, sqrtf(2.0f / (9.0f * kCin[l])));
        for (long long i = 0; i < n->L[l].nw; ++i) h[(size_t)(n->L[l].woff + i)] = nd(rng);
    }
    std::normal_distribution<float> hd(0.0f, 0.01f);
    for (int c = 0; c < 32; ++c) h[(size_t)(n->whoff + c)] = hd(rng);
    if ((e = cudaMemcpyAsync(n->params, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(n->grads, 0, sizeof(float) * off, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(n->m, 0, sizeof(float) * off, st)) != cudaSuccess ||
        (e = cudaMemsetAsync(n->v, 0, sizeof(float) * off, st)) != cudaSuccess) {
        delete n;
        return e;
    }
    for (int l = 1; l < 14; ++l) {
        Layer &L = n->L[l];
        if ((e = weights_bf16(n->params + L.woff, L.nw, L.wbf, L.wtbf, L.cout, L.cin, st)) != cudaSuccess) {
            delete n;
            return e;
        }
    }
    // the host vector is staged before cudaMemcpyAsync returns; wait anyway so
    // the network is ready when the constructor returns
    if ((e = cudaStreamSynchronize(st)) != cudaSuccess) {
        delete n;
        return e;
    }
    *out = n;
    return cudaSuccess;
}

void net_free(Net *n) { delete n; }
long long net_nparams(const Net *n) { return n->nparams; }
float *net_params(Net *n) { return n->params; }
float *net_grads(Net *n) { return n->grads; }
float *net_adam_m(Net *n) { return n->m; }
float *net_adam_v(Net *n) { return n->v; }
int *net_adam_step(Net *n) { return &n->step; }

cudaError_t net_refresh_weights(Net *n, cudaStream_t st) {
    for (int l = 1; l < 14; ++l) {
        Layer &L = n->L[l];
        NET_TRY(weights_bf16(n->params + L.woff, L.nw, L.wbf, L.wtbf, L.cout, L.cin, st));
    }
    return cudaSuccess;
}

static cudaError_t conv(const Net *n, int l, int B, const uint16_t *x, int ldx, int xoff, uint16_t *y, int ldy,
                        int yoff, int *err, unsigned long long lim, cudaStream_t st) {
    const Layer &L = n->L[l];
    const int S = n->N >> kLevel[l];
    ConvArgs c = {x, ldx, xoff, L.cin, B, S, S, L.wbf, n->params + L.boff, y, ldy, yoff, L.cout, nullptr, 0, 0};
    return conv3x3(c, EPI_BIAS_RELU, err, lim, st);
}

cudaError_t net_forward(Net *n, int B, const float *x, float *y, const float *target, int *err,
                        unsigned long long lim, cudaStream_t st) {
    if (B < 1 || B > n->maxB) return cudaErrorInvalidValue;
    const int N = n->N, N2 = N / 2, N4 = N / 4, N8 = N / 8;
    const long long P0 = (long long)B * N * N;
    NET_TRY(cudaMemcpyAsync(n->x0, x, sizeof(float) * P0, cudaMemcpyDeviceToDevice, st));
    NET_TRY(first_conv(n->x0, n->params + n->L[0].woff, n->params + n->L[0].boff, n->e1a, B, N, N, 32, 32, st));
    NET_TRY(conv(n, 1, B, n->e1a, 32, 0, n->cat1, 96, 64, err, lim, st));
    NET_TRY(maxpool(n->cat1, 96, 64, n->p1, 32, B, N, N, 32, st));
    NET_TRY(conv(n, 2, B, n->p1, 32, 0, n->e2a, 64, 0, err, lim, st));
    NET_TRY(conv(n, 3, B, n->e2a, 64, 0, n->cat2, 192, 128, err, lim, st));
    NET_TRY(maxpool(n->cat2, 192, 128, n->p2, 64, B, N2, N2, 64, st));
    NET_TRY(conv(n, 4, B, n->p2, 64, 0, n->e3a, 128, 0, err, lim, st));
    NET_TRY(conv(n, 5, B, n->e3a, 128, 0, n->cat3, 384, 256, err, lim, st));
    NET_TRY(maxpool(n->cat3, 384, 256, n->p3, 128, B, N4, N4, 128, st));
    NET_TRY(conv(n, 6, B, n->p3, 128, 0, n->e4a, 256, 0, err, lim, st));
    NET_TRY(conv(n, 7, B, n->e4a, 256, 0, n->e4, 256, 0, err, lim, st));
    NET_TRY(upsample(n->e4, 256, n->cat3, 384, 0, B, N4, N4, 256, st));
    NET_TRY(conv(n, 8, B, n->cat3, 384, 0, n->d3a, 128, 0, err, lim, st));
    NET_TRY(conv(n, 9, B, n->d3a, 128, 0, n->d3, 128, 0, err, lim, st));
    NET_TRY(upsample(n->d3, 128, n->cat2, 192, 0, B, N2, N2, 128, st));
    NET_TRY(conv(n, 10, B, n->cat2, 192, 0, n->d2a, 64, 0, err, lim, st));
    NET_TRY(conv(n, 11, B, n->d2a, 64, 0, n->d2, 64, 0, err, lim, st));
    NET_TRY(upsample(n->d2, 64, n->cat1, 96, 0, B, N, N, 64, st));
    NET_TRY(conv(n, 12, B, n->cat1, 96, 0, n->d1a, 32, 0, err, lim, st));
    NET_TRY(conv(n, 13, B, n->d1a, 32, 0, n->d1, 32, 0, err, lim, st));
    (void)N8;
    if (target) {
        NET_TRY(cudaMemcpyAsync(n->tgt, target, sizeof(float) * P0, cudaMemcpyDeviceToDevice, st));
        NET_TRY(cudaMemsetAsync(n->loss, 0, sizeof(double), st));
    }
    return head(n->x0, n->d1, 32, n->params + n->whoff, n->params + n->bhoff, y, target ? n->tgt : nullptr, n->g,
                n->loss, P0, 32, st);
}

// Backward of 3x3 layer l: bias and weight gradients from dz (BF16 NHWC,
// ld = cout) and the layer input x; with dx, the input gradient masked by x > 0.
static cudaError_t layer_bwd(Net *n, int l, int B, const uint16_t *x, int ldx, int xoff, const uint16_t *dz,
                             uint16_t *dx, int *err, unsigned long long lim, cudaStream_t st) {
    const Layer &L = n->L[l];
    const int S = n->N >> kLevel[l];
    const long long P = (long long)B * S * S;
    NET_TRY(bias_grad(dz, L.cout, n->grads + L.boff, P, L.cout, st));
    NET_TRY(to_cmajor(dz, L.cout, 0, n->dzT, L.cout, P, S, 0, st));
    NET_TRY(to_cmajor(x, ldx, xoff, n->xT3, L.cin, P, S, 1, st));
    const int mt = (L.cout + 127) / 128;
    const int nt = L.cin <= 256 ? 1 : L.cin / (L.cin % 192 == 0 ? 192 : 128);
    const long long chunks = P / (S >= 64 ? 64 : 32);
    long long ks = (152LL * 2) / (9LL * mt * nt);
    if (ks < 1) ks = 1;
    if (ks > chunks) ks = chunks;
    WgradArgs w = {n->dzT, n->xT3, n->grads + L.woff, L.cin, L.cout, B, S, S, (int)ks};
    NET_TRY(conv3x3_wgrad(w, err, lim, st));
    if (dx) {
        ConvArgs c = {dz, L.cout, 0, L.cout, B, S, S, L.wtbf, nullptr, dx, L.cin, 0, L.cin, x, ldx, xoff};
        NET_TRY(conv3x3(c, EPI_MASK, err, lim, st));
    }
    return cudaSuccess;
}

cudaError_t net_backward(Net *n, int B, int *err, unsigned long long lim, cudaStream_t st) {
    const int N = n->N, N2 = N / 2, N4 = N / 4, N8 = N / 8;
    const long long P0 = (long long)B * N * N;
    uint16_t **gA = n->gA, **gB = n->gB;
    NET_TRY(head_bwd(n->g, n->d1, 32, n->params + n->whoff, gA[0], 32, n->grads + n->whoff, n->grads + n->bhoff, P0,
                     32, st));
    NET_TRY(layer_bwd(n, 13, B, n->d1a, 32, 0, gA[0], gB[0], err, lim, st));
    NET_TRY(layer_bwd(n, 12, B, n->cat1, 96, 0, gB[0], n->gcat1, err, lim, st));
    NET_TRY(upsample_bwd(n->gcat1, 96, 0, gA[1], 64, B, N2, N2, 64, st));
    NET_TRY(layer_bwd(n, 11, B, n->d2a, 64, 0, gA[1], gB[1], err, lim, st));
    NET_TRY(layer_bwd(n, 10, B, n->cat2, 192, 0, gB[1], n->gcat2, err, lim, st));
    NET_TRY(upsample_bwd(n->gcat2, 192, 0, gA[2], 128, B, N4, N4, 128, st));
    NET_TRY(layer_bwd(n, 9, B, n->d3a, 128, 0, gA[2], gB[2], err, lim, st));
    NET_TRY(layer_bwd(n, 8, B, n->cat3, 384, 0, gB[2], n->gcat3, err, lim, st));
    NET_TRY(upsample_bwd(n->gcat3, 384, 0, gA[3], 256, B, N8, N8, 256, st));
    NET_TRY(layer_bwd(n, 7, B, n->e4a, 256, 0, gA[3], gB[3], err, lim, st));
    NET_TRY(layer_bwd(n, 6, B, n->p3, 128, 0, gB[3], gA[3], err, lim, st));             // dP3 (128 ch) in gA[3]
    NET_TRY(maxpool_bwd(n->cat3, 384, 256, gA[3], 128, n->gcat3, 384, 256, gA[2], 128, B, N4, N4, 128, st));
    NET_TRY(layer_bwd(n, 5, B, n->e3a, 128, 0, gA[2], gB[2], err, lim, st));
    NET_TRY(layer_bwd(n, 4, B, n->p2, 64, 0, gB[2], gA[2], err, lim, st));              // dP2 (64 ch) in gA[2]
    NET_TRY(maxpool_bwd(n->cat2, 192, 128, gA[2], 64, n->gcat2, 192, 128, gA[1], 64, B, N2, N2, 64, st));
    NET_TRY(layer_bwd(n, 3, B, n->e2a, 64, 0, gA[1], gB[1], err, lim, st));
    NET_TRY(layer_bwd(n, 2, B, n->p1, 32, 0, gB[1], gA[1], err, lim, st));              // dP1 (32 ch) in gA[1]
    NET_TRY(maxpool_bwd(n->cat1, 96, 64, gA[1], 32, n->gcat1, 96, 64, gA[0], 32, B, N, N, 32, st));
    NET_TRY(layer_bwd(n, 1, B, n->e1a, 32, 0, gA[0], gB[0], err, lim, st));
    return first_conv_wgrad(n->x0, gB[0], 32, n->grads + n->L[0].woff, n->grads + n->L[0].boff, B, N, N, 32, st);
}

cudaError_t net_adam(Net *n, float lr, cudaStream_t st) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    n->step += 1;
    for (int l = 0; l < 14; ++l) {
        Layer &L = n->L[l];
        NET_TRY(adam(n->params + L.woff, n->grads + L.woff, n->m + L.woff, n->v + L.woff, L.nw, lr, b1, b2, eps,
                     n->step, l > 0 ? L.wbf : nullptr, l > 0 ? L.wtbf : nullptr, L.cout, L.cin, st));
        NET_TRY(adam(n->params + L.boff, n->grads + L.boff, n->m + L.boff, n->v + L.boff, L.cout, lr, b1, b2, eps,
                     n->step, nullptr, nullptr, 0, 0, st));
    }
    return adam(n->params + n->whoff, n->grads + n->whoff, n->m + n->whoff, n->v + n->whoff, 33, lr, b1, b2, eps,
                n->step, nullptr, nullptr, 0, 0, st);
}

double *net_loss(Net *n) { return n->loss; }

}  // namespace unet
}  // namespace synk

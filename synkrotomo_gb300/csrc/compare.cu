// The reference's validation programs on the GPU (futhark/tools/diff.fut,
// mse.fut, sanityCheck.fut): one pass over two float32 arrays that yields
//   count  the indices i > 0 with |sane[i] - test[i]| > tol      (diff.fut:4-6)
//   sse    the sum of (sane[i] - test[i])^2, accumulated in FP64  (mse.fut:2-3)
//   all_ok whether |sane[i] - test[i]| < tol for every i          (sanityCheck.fut:3-4)
// diff.fut marks the indices that pass with -1 and keeps those > 0, so index 0
// is never counted; that is kept.  A NaN difference is neither counted by diff
// nor accepted by sanityCheck, as the comparisons of the reference decide.
//
// HBM-bound: 8 bytes per element.  A grid of whole waves (SMs x 4 blocks of
// 256 threads) strides over float4 pairs when both arrays are 16-byte aligned;
// block partials are reduced in shared memory and added with one atomic each.
#include <algorithm>

#include "synk_internal.cuh"

namespace synk {

namespace {

struct CmpAcc {
    unsigned long long count = 0;
    double sse = 0.0;
    int ok = 1;
};

__device__ __forceinline__ void cmp_one(float s, float t, long long i, float tol, CmpAcc &a) {
    const float d = fabsf(s - t);
    if (d > tol && i > 0) ++a.count;
    if (!(d < tol)) a.ok = 0;
    const double dd = (double)s - (double)t;
    a.sse = fma(dd, dd, a.sse);
}

__global__ void __launch_bounds__(256) compare_kernel(const float *__restrict__ sane, const float *__restrict__ test,
                                                      long long n, float tol, int vec, CompareResult *out) {
    CmpAcc a;
    const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    const long long nth = (long long)gridDim.x * blockDim.x;
    long long done = 0;
    if (vec) {
        const long long n4 = n >> 2;
        const float4 *s4 = reinterpret_cast<const float4 *>(sane);
        const float4 *t4 = reinterpret_cast<const float4 *>(test);
        for (long long j = tid; j < n4; j += nth) {
            const float4 s = __ldcs(s4 + j), t = __ldcs(t4 + j);
            cmp_one(s.x, t.x, 4 * j, tol, a);
            cmp_one(s.y, t.y, 4 * j + 1, tol, a);
            cmp_one(s.z, t.z, 4 * j + 2, tol, a);
            cmp_one(s.w, t.w, 4 * j + 3, tol, a);
        }
        done = n4 << 2;
    }
    for (long long i = done + tid; i < n; i += nth) cmp_one(__ldcs(sane + i), __ldcs(test + i), i, tol, a);

    for (int o = 16; o; o >>= 1) {
        a.count += __shfl_xor_sync(0xffffffffu, a.count, o);
        a.sse += __shfl_xor_sync(0xffffffffu, a.sse, o);
    }
    a.ok = __all_sync(0xffffffffu, a.ok);
    __shared__ unsigned long long sc[8];
    __shared__ double ss[8];
    __shared__ int so[8];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) {
        sc[w] = a.count;
        ss[w] = a.sse;
        so[w] = a.ok;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long c = 0;
        double s = 0.0;
        int ok = 1;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
            c += sc[k];
            s += ss[k];
            ok &= so[k];
        }
        if (c) atomicAdd(reinterpret_cast<unsigned long long *>(&out->count), c);
        atomicAdd(&out->sse, s);
        if (!ok) atomicAnd(&out->all_ok, 0);
    }
}

__global__ void compare_init_kernel(CompareResult *out) {
    out->count = 0;
    out->sse = 0.0;
    out->all_ok = 1;
}

// diff.fut returns an i32 count, mse.fut an f32 mean, sanityCheck.fut a bool.
__global__ void compare_finish_kernel(const CompareResult *r, long long n, int what, void *dst) {
    if (what == 0) *reinterpret_cast<int *>(dst) = (int)r->count;
    else if (what == 1) *reinterpret_cast<float *>(dst) = n ? (float)(r->sse / (double)n) : __int_as_float(0x7fc00000);
    else *reinterpret_cast<unsigned char *>(dst) = (unsigned char)(r->all_ok != 0);
}

}  // namespace

cudaError_t launch_compare(const float *sane, const float *test, long long n, float tol, CompareResult *out,
                           cudaStream_t stream) {
    compare_init_kernel<<<1, 1, 0, stream>>>(out);
    if (n > 0) {
        int sms = 0, dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const long long want = (n / 4 + 255) / 256;
        const int grid = (int)std::max(1LL, std::min<long long>(want, (long long)sms * 4));
        const int vec = ((reinterpret_cast<uintptr_t>(sane) | reinterpret_cast<uintptr_t>(test)) & 15) == 0;
        compare_kernel<<<grid, 256, 0, stream>>>(sane, test, n, tol, vec, out);
    }
    return cudaGetLastError();
}

cudaError_t launch_compare_finish(const CompareResult *r, long long n, int what, void *dst, cudaStream_t stream) {
    compare_finish_kernel<<<1, 1, 0, stream>>>(r, n, what, dst);
    return cudaGetLastError();
}

}  // namespace synk

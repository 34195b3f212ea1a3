// C ABI of libsynk (declared in include/synk.h): contexts, argument checks,
// scratch memory and the entry points of the reference programs.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include "synk_internal.cuh"
#include "sirt_internal.cuh"

using namespace synk;

struct synk_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int *d_status = nullptr;   // written by persistent kernels (SYNK_ETIMEOUT)
    unsigned long long barrier_timeout_ns = 2000000000ull;
};

namespace {

int fail(synk_context *ctx, int code, const char *fmt, ...) __attribute__((format(printf, 3, 4)));
int fail(synk_context *ctx, int code, const char *fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    if (ctx) ctx->err = buf;
    return code;
}

int cuda_fail(synk_context *ctx, cudaError_t e, const char *what) {
    return fail(ctx, e == cudaErrorMemoryAllocation ? SYNK_ENOMEM : SYNK_ECUDA, "%s: %s", what,
                cudaGetErrorString(e));
}

#define SYNK_CUDA(call, what)                                   \
    do {                                                        \
        cudaError_t e_ = (call);                                \
        if (e_ != cudaSuccess) return cuda_fail(ctx, e_, what); \
    } while (0)

// Stream-ordered scratch memory, released on the same stream when it goes out
// of scope (the frees are ordered after every kernel enqueued before them).
struct Scratch {
    cudaStream_t st;
    std::vector<void *> ptrs;
    explicit Scratch(cudaStream_t s) : st(s) {}
    ~Scratch() {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
    template <class T>
    cudaError_t get(T **out, size_t count) {
        void *p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, count * sizeof(T) + 16, st);
        if (e != cudaSuccess) return e;
        ptrs.push_back(p);
        *out = static_cast<T *>(p);
        return cudaSuccess;
    }
};

int64_t isqrt64(int64_t n) {
    if (n < 0) return -1;
    int64_t r = (int64_t)sqrt((double)n);
    while (r * r > n) --r;
    while ((r + 1) * (r + 1) <= n) ++r;
    return r;
}

// rhosprpixel = ceil(sqrt(2)/deltarho) in f32 (backprojection.fut:87).
int rhos_per_pixel(float deltarho) { return (int)ceilf(sqrtf(2.0f) / deltarho); }

constexpr int kMaxSize = 16384;      // image side (the traversal's floor needs |x| < 2^22)
constexpr int64_t kMaxDet = 1 << 22; // detectors per angle

int check_ctx(synk_context *ctx) {
    if (!ctx) return SYNK_EINVAL;
    cudaError_t e = cudaSetDevice(ctx->device);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
    ctx->err.clear();
    return SYNK_OK;
}

int check_geometry(synk_context *ctx, int64_t a, float rhozero, float deltarho, int64_t numrhos, int64_t size) {
    if (a < 1) return fail(ctx, SYNK_EINVAL, "need at least one angle (got %lld)", (long long)a);
    if (a > (1 << 24)) return fail(ctx, SYNK_EINVAL, "too many angles (%lld)", (long long)a);
    if (numrhos < 1 || numrhos > kMaxDet)
        return fail(ctx, SYNK_EINVAL, "numrhos must be in [1, %lld] (got %lld)", (long long)kMaxDet, (long long)numrhos);
    if (size < 2 || size > kMaxSize || (size & 1))
        return fail(ctx, SYNK_EINVAL, "image side must be even and in [2, %d] (got %lld)", kMaxSize, (long long)size);
    if (!isfinite(rhozero)) return fail(ctx, SYNK_EINVAL, "rhozero must be finite");
    if (!(deltarho > 0.0f) || !isfinite(deltarho))
        return fail(ctx, SYNK_EINVAL, "deltarho must be positive and finite (got %g)", (double)deltarho);
    if (rhos_per_pixel(deltarho) > 64) return fail(ctx, SYNK_EINVAL, "deltarho too small (%g)", (double)deltarho);
    // detector positions and indices must stay well inside the range where the
    // kernels' float32 floor/ceil are exact (|x| < 2^22)
    const double last = (double)rhozero + (double)(numrhos - 1) * deltarho;
    if (fabs((double)rhozero) > 1.0e6 || fabs(last) > 1.0e6 || fabs((double)rhozero) / deltarho > 2.0e6)
        return fail(ctx, SYNK_EINVAL, "detector range [%g, %g] too large", (double)rhozero, last);
    return SYNK_OK;
}

ProbGeom make_geom(int64_t a, float rhozero, float deltarho, int64_t numrhos, int64_t size, const AngleGeom *geom) {
    ProbGeom P;
    P.N = (int)size;
    P.half = (int)size / 2;
    P.a = (int)a;
    P.D = (int)numrhos;
    P.rpp = rhos_per_pixel(deltarho);
    P.rhozero = rhozero;
    P.deltarho = deltarho;
    P.inv_deltarho = 1.0f / deltarho;
    P.geom = geom;
    return P;
}

int image_side(synk_context *ctx, int64_t n, int64_t *size) {
    const int64_t s = isqrt64(n);
    if (s < 0 || s * s != n)
        return fail(ctx, SYNK_EINVAL, "image length %lld is not a square number of pixels", (long long)n);
    *size = s;
    return SYNK_OK;
}

int pick_split(long long tasks, long long resident_warps, int max_split) {
    int s = 1;
    while (s < max_split && tasks * s < 2 * resident_warps) s *= 2;
    return s;
}

int forward(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero, float deltarho,
            int32_t numrhos, const float *image, int64_t n) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out || !angles || !image) return fail(ctx, SYNK_EINVAL, "null array pointer");
    int64_t size = 0;
    if ((rc = image_side(ctx, n, &size))) return rc;
    if ((rc = check_geometry(ctx, a, rhozero, deltarho, numrhos, size))) return rc;
    Scratch sc(ctx->stream);
    AngleGeom *geom;
    float *imgT;
    SYNK_CUDA(sc.get(&geom, (size_t)a), "cudaMallocAsync(geometry)");
    SYNK_CUDA(sc.get(&imgT, (size_t)n), "cudaMallocAsync(transposed image)");
    SYNK_CUDA(launch_geometry(angles, (int)a, geom, ctx->stream), "geometry kernel");
    SYNK_CUDA(launch_transpose(image, imgT, (int)size, 1, ctx->stream), "transpose kernel");
    const ProbGeom P = make_geom(a, rhozero, deltarho, numrhos, size, geom);
    SYNK_CUDA(launch_fp(P, image, imgT, out, ctx->stream), "forward projection kernel");
    return SYNK_OK;
}

int backward(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero, float deltarho,
             int32_t size_in, const float *projections, int64_t p) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out || !angles || !projections) return fail(ctx, SYNK_EINVAL, "null array pointer");
    if (a < 1) return fail(ctx, SYNK_EINVAL, "need at least one angle (got %lld)", (long long)a);
    if (p < a || p % a) return fail(ctx, SYNK_EINVAL, "projection length %lld is not a multiple of %lld angles",
                                    (long long)p, (long long)a);
    const int64_t numrhos = p / a;
    if ((rc = check_geometry(ctx, a, rhozero, deltarho, numrhos, size_in))) return rc;
    Scratch sc(ctx->stream);
    AngleGeom *geom;
    SYNK_CUDA(sc.get(&geom, (size_t)a), "cudaMallocAsync(geometry)");
    SYNK_CUDA(launch_geometry(angles, (int)a, geom, ctx->stream), "geometry kernel");
    const ProbGeom P = make_geom(a, rhozero, deltarho, numrhos, size_in, geom);
    SYNK_CUDA(launch_bp(P, projections, out, ctx->stream), "backprojection kernel");
    return SYNK_OK;
}

__global__ void fill_i32_kernel(int *p, int n, int v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

int sirt_slices(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero, float deltarho,
                int64_t numrhos, int64_t size, int64_t nslices, const float *image, const float *projections,
                int32_t iterations, const synk_sirt_options *opts) {
    int rc;
    if (!out || !angles || !projections) return fail(ctx, SYNK_EINVAL, "null array pointer");
    if ((rc = check_geometry(ctx, a, rhozero, deltarho, numrhos, size))) return rc;
    if (nslices < 1 || nslices > (1 << 20)) return fail(ctx, SYNK_EINVAL, "bad slice count %lld", (long long)nslices);
    if (iterations < 0) return fail(ctx, SYNK_EINVAL, "iterations must be >= 0 (got %d)", iterations);
    const size_t n = (size_t)size * size, pr = (size_t)a * numrhos;
    if ((double)nslices * (double)(n > pr ? n : pr) > 2.0e9 * 4)
        return fail(ctx, SYNK_EINVAL, "slice stack too large");
    cudaStream_t st = ctx->stream;
    // start image
    if (image) SYNK_CUDA(cudaMemcpyAsync(out, image, sizeof(float) * n * nslices, cudaMemcpyDeviceToDevice, st), "copy start");
    else SYNK_CUDA(cudaMemsetAsync(out, 0, sizeof(float) * n * nslices, st), "zero start");
    if (iterations == 0 && !(opts && opts->residuals)) {
        if (opts && opts->iterations_done) SYNK_CUDA(cudaMemsetAsync(opts->iterations_done, 0, sizeof(int) * nslices, st), "memset");
        return SYNK_OK;
    }
    Scratch sc(st);
    AngleGeom *geom;
    float *R, *C, *xT, *rr;
    double *res2, *b2;
    int *stop_iter;
    unsigned *words;
    const size_t K = (size_t)iterations + 1;
    SYNK_CUDA(sc.get(&geom, (size_t)a), "cudaMallocAsync");
    SYNK_CUDA(sc.get(&R, pr), "cudaMallocAsync(R)");
    SYNK_CUDA(sc.get(&C, n), "cudaMallocAsync(C)");
    SYNK_CUDA(sc.get(&xT, n * nslices), "cudaMallocAsync(xT)");
    SYNK_CUDA(sc.get(&rr, pr * nslices), "cudaMallocAsync(residual)");
    SYNK_CUDA(sc.get(&res2, K * nslices), "cudaMallocAsync");
    SYNK_CUDA(sc.get(&b2, (size_t)nslices), "cudaMallocAsync");
    SYNK_CUDA(sc.get(&stop_iter, (size_t)nslices), "cudaMallocAsync");
    SYNK_CUDA(sc.get(&words, 8), "cudaMallocAsync");
    SYNK_CUDA(cudaMemsetAsync(res2, 0, sizeof(double) * K * nslices, st), "memset");
    SYNK_CUDA(cudaMemsetAsync(b2, 0, sizeof(double) * nslices, st), "memset");
    SYNK_CUDA(cudaMemsetAsync(words, 0, sizeof(unsigned) * 8, st), "memset");
    fill_i32_kernel<<<(unsigned)((nslices + 255) / 256), 256, 0, st>>>(stop_iter, (int)nslices, 0x7fffffff);
    SYNK_CUDA(cudaGetLastError(), "fill kernel");
    SYNK_CUDA(launch_geometry(angles, (int)a, geom, st), "geometry kernel");
    const ProbGeom P = make_geom(a, rhozero, deltarho, numrhos, size, geom);
    SYNK_CUDA(launch_normalisers(P, R, C, st), "normaliser kernels");
    SYNK_CUDA(launch_transpose(out, xT, (int)size, (int)nslices, st), "transpose kernel");
    SYNK_CUDA(launch_sumsq(projections, pr, (int)nslices, b2, st), "norm kernel");

    SirtParams sp;
    sp.P = P;
    sp.R = R;
    sp.C = C;
    sp.b = projections;
    sp.x = out;
    sp.xT = xT;
    sp.rr = rr;
    sp.res2 = res2;
    sp.b2 = b2;
    sp.stop_iter = stop_iter;
    sp.bar = words;
    sp.work = words + 4;
    sp.status = ctx->d_status;
    sp.timeout_ns = ctx->barrier_timeout_ns;
    sp.tol2 = (opts && opts->tol > 0.0) ? opts->tol * opts->tol : 0.0;
    sp.nslices = (int)nslices;
    sp.iterations = iterations;
    sp.record_final = (opts && opts->residuals) ? 1 : 0;
    int bps = 0;
    const int grid = sirt_persistent_grid(&bps);
    if (grid < 1) return fail(ctx, SYNK_ECUDA, "persistent SIRT kernel cannot be resident");
    const long long resident_warps = (long long)grid * 8;
    const long long fp_tasks = (long long)nslices * a * ((numrhos + 31) / 32);
    const long long bp_tasks = (long long)nslices * size * ((size + 31) / 32);
    int fs = opts && opts->fp_split > 0 ? opts->fp_split : pick_split(fp_tasks, resident_warps, (int)(size / 16 > 8 ? 8 : (size / 16 < 1 ? 1 : size / 16)));
    int bs = opts && opts->bp_split > 0 ? opts->bp_split : pick_split(bp_tasks, resident_warps, (int)(a / 8 > 8 ? 8 : (a / 8 < 1 ? 1 : a / 8)));
    if (fs != 1 && fs != 2 && fs != 4 && fs != 8) return fail(ctx, SYNK_EINVAL, "fp_split must be 1, 2, 4 or 8");
    if (bs != 1 && bs != 2 && bs != 4 && bs != 8) return fail(ctx, SYNK_EINVAL, "bp_split must be 1, 2, 4 or 8");
    sp.fp_split = fs;
    sp.bp_split = bs;
    SYNK_CUDA(launch_sirt_persistent(sp, grid, st), "persistent SIRT kernel");
    if (opts && (opts->residuals || opts->iterations_done))
        SYNK_CUDA(launch_sirt_finalize(sp, opts->residuals, opts->iterations_done, st), "finalize kernel");
    return SYNK_OK;
}

}  // namespace

extern "C" {

const char *synk_version(void) { return "synkrotomo-gb300 0.1 (sm_103a)"; }

int synk_context_new(synk_context **out, int device, void *stream) {
    if (!out) return SYNK_EINVAL;
    *out = nullptr;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return SYNK_ECUDA;
    if (device < 0 || device >= ndev) return SYNK_EINVAL;
    if (cudaSetDevice(device) != cudaSuccess) return SYNK_ECUDA;
    synk_context *ctx = new synk_context();
    ctx->device = device;
    ctx->stream = static_cast<cudaStream_t>(stream);
    if (cudaMalloc(&ctx->d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(ctx->d_status, 0, sizeof(int)) != cudaSuccess) {
        delete ctx;
        return SYNK_ENOMEM;
    }
    *out = ctx;
    return SYNK_OK;
}

void synk_context_free(synk_context *ctx) {
    if (!ctx) return;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    cudaFree(ctx->d_status);
    delete ctx;
}

int synk_context_set_stream(synk_context *ctx, void *stream) {
    if (!ctx) return SYNK_EINVAL;
    ctx->stream = static_cast<cudaStream_t>(stream);
    return SYNK_OK;
}

int synk_context_sync(synk_context *ctx) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    SYNK_CUDA(cudaStreamSynchronize(ctx->stream), "cudaStreamSynchronize");
    int status = 0;
    SYNK_CUDA(cudaMemcpy(&status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost), "read status");
    if (status != SYNK_OK) {
        cudaMemset(ctx->d_status, 0, sizeof(int));
        if (status == SYNK_ETIMEOUT)
            return fail(ctx, SYNK_ETIMEOUT, "a grid barrier of the persistent SIRT kernel timed out; the result is invalid");
        return fail(ctx, status, "device status %d", status);
    }
    return SYNK_OK;
}

const char *synk_context_get_error(synk_context *ctx) { return ctx ? ctx->err.c_str() : "null context"; }

int synk_forwardprojection(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                           float deltarho, int32_t numrhos, const float *image, int64_t n) {
    return forward(ctx, out, angles, a, rhozero, deltarho, numrhos, image, n);
}

int synk_forwardprojection_sparse(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                                  float deltarho, int32_t numrhos, const float *image, int64_t n) {
    return forward(ctx, out, angles, a, rhozero, deltarho, numrhos, image, n);
}

int synk_backprojection(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                        float deltarho, int32_t size, const float *projections, int64_t p) {
    return backward(ctx, out, angles, a, rhozero, deltarho, size, projections, p);
}

int synk_backprojection_sparse(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                               float deltarho, int32_t size, const float *projections, int64_t p) {
    return backward(ctx, out, angles, a, rhozero, deltarho, size, projections, p);
}

int synk_SIRT(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero, float deltarho,
              const float *image, int64_t n, const float *projections, int64_t p, int32_t iterations) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!image) return fail(ctx, SYNK_EINVAL, "null array pointer");
    int64_t size = 0;
    if ((rc = image_side(ctx, n, &size))) return rc;
    if (a < 1) return fail(ctx, SYNK_EINVAL, "need at least one angle (got %lld)", (long long)a);
    if (p < a || p % a) return fail(ctx, SYNK_EINVAL, "projection length %lld is not a multiple of %lld angles",
                                    (long long)p, (long long)a);
    return sirt_slices(ctx, out, angles, a, rhozero, deltarho, p / a, size, 1, image, projections, iterations, nullptr);
}

int synk_SIRT3D(synk_context *ctx, float *out, const float *angles, int64_t a, const float *rhos, int64_t r,
                const float *projections, int64_t p, int32_t iterations, int32_t size) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!rhos) return fail(ctx, SYNK_EINVAL, "null array pointer");
    if (r < 2) return fail(ctx, SYNK_EINVAL, "rhos needs at least two detector positions (got %lld)", (long long)r);
    if (size < 1) return fail(ctx, SYNK_EINVAL, "size must be positive (got %d)", size);
    if (p != (int64_t)size * a * r)
        return fail(ctx, SYNK_EINVAL, "projections has %lld values, expected size*a*r = %lld", (long long)p,
                    (long long)size * a * r);
    float rh[2];
    SYNK_CUDA(cudaMemcpyAsync(rh, rhos, sizeof rh, cudaMemcpyDeviceToHost, ctx->stream), "read rhos");
    SYNK_CUDA(cudaStreamSynchronize(ctx->stream), "read rhos");
    const float rhozero = rh[0];
    const float deltarho = rh[1] - rh[0];
    return sirt_slices(ctx, out, angles, a, rhozero, deltarho, r, size, size, nullptr, projections, iterations, nullptr);
}

int synk_sirt_slices(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                     float deltarho, int32_t numrhos, int32_t size, int32_t nslices, const float *image,
                     const float *projections, int32_t iterations, const synk_sirt_options *opts) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    return sirt_slices(ctx, out, angles, a, rhozero, deltarho, numrhos, size, nslices, image, projections,
                       iterations, opts);
}

}  // extern "C"

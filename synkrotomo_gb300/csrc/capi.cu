// C ABI of libsynk (declared in include/synk.h): contexts, argument checks,
// scratch memory and the entry points of the reference programs.
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <climits>
#include <mutex>
#include <string>
#include <vector>

#include "synk_internal.cuh"
#include "sirt_internal.cuh"
#include "csr_internal.cuh"
#include "fp_tile.cuh"
#include "bp_tile.cuh"
#include "umma_gemm.cuh"
#include "unet.cuh"

using namespace synk;

struct synk_csr {
    int device = 0;
    int64_t rows = 0, cols = 0, nnz = 0;
    int64_t *ptr = nullptr, *ptr_t = nullptr;
    int *idx = nullptr, *idx_t = nullptr;
    float *vals = nullptr, *vals_t = nullptr;
};

struct synk_context {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string err;
    int *d_status = nullptr;   // written by persistent kernels (SYNK_ETIMEOUT)
    int *h_poll = nullptr;     // pinned: active-slice counts read back by the SIRT loop's stopping rule
    cudaEvent_t poll_ev[2] = {nullptr, nullptr};
    unsigned long long barrier_timeout_ns = 2000000000ull;
    unsigned barrier_extra = 0;   // fault injection: blocks a grid barrier waits for that never come
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
// reserve() takes one block that later get() calls carve (256-byte aligned),
// so a call with several small buffers costs one allocation and one free.
struct Scratch {
    cudaStream_t st;
    std::vector<void *> ptrs;
    char *arena = nullptr;
    size_t arena_left = 0;
    explicit Scratch(cudaStream_t s) : st(s) {}
    ~Scratch() {
        for (void *p : ptrs) cudaFreeAsync(p, st);
    }
    static size_t round(size_t b) { return (b + 16 + 255) / 256 * 256; }
    cudaError_t reserve(size_t bytes) {
        void *p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, bytes, st);
        if (e != cudaSuccess) return e;
        ptrs.push_back(p);
        arena = static_cast<char *>(p);
        arena_left = bytes;
        return cudaSuccess;
    }
    template <class T>
    cudaError_t get(T **out, size_t count) {
        const size_t need = round(count * sizeof(T));
        if (need <= arena_left) {
            *out = reinterpret_cast<T *>(arena);
            arena += need;
            arena_left -= need;
            return cudaSuccess;
        }
        void *p = nullptr;
        cudaError_t e = cudaMallocAsync(&p, count * sizeof(T) + 16, st);
        if (e != cudaSuccess) return e;
        ptrs.push_back(p);
        *out = static_cast<T *>(p);
        return cudaSuccess;
    }
};

// scratch bytes of the angle lists (make_lists)
size_t lists_bytes(int64_t a) {
    return Scratch::round(sizeof(int) * ((size_t)a + 64)) + Scratch::round(sizeof(int) * (size_t)a) +
           Scratch::round(sizeof(int) * 4);
}

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
    // the detector nearest rho = 0: zi = round(-rhozero/deltarho), rz_c its
    // position (exact in f32 for deltarho = 1: rhozero + an integer)
    const double zi = nearbyint(-(double)rhozero / (double)deltarho);
    P.zi = (int)zi;
    P.rz_c = (float)((double)rhozero + zi * (double)deltarho);
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

// Angle lists of a geometry in scratch memory: order[a + 64], exact[a], counts[3].
// Geometry table and angle lists of P (P.geom must point at scratch of a
// entries) in one setup launch; with x given, the same launch writes the pair
// images of x for the forward projector.
cudaError_t make_setup(Scratch &sc, const float *angles, const ProbGeom &P, AngleLists *L, cudaStream_t st,
                       const float *x = nullptr, float2 *xpair = nullptr, float2 *xTpair = nullptr) {
    int *order, *exact, *counts;
    cudaError_t e;
    if ((e = sc.get(&order, (size_t)P.a + 64)) != cudaSuccess) return e;
    if ((e = sc.get(&exact, (size_t)P.a)) != cudaSuccess) return e;
    if ((e = sc.get(&counts, 4)) != cudaSuccess) return e;
    if ((e = launch_setup(angles, P.a, const_cast<AngleGeom *>(P.geom), order, exact, counts, x, xpair, xTpair, P.N,
                          st)) != cudaSuccess)
        return e;
    L->order = order;
    L->exact = exact;
    L->counts = counts;
    return cudaSuccess;
}

int forward(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero, float deltarho,
            int32_t numrhos, const float *image, int64_t n) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out || !angles || !image) return fail(ctx, SYNK_EINVAL, "null array pointer");
    int64_t size = 0;
    if ((rc = image_side(ctx, n, &size))) return rc;
    if ((rc = check_geometry(ctx, a, rhozero, deltarho, numrhos, size))) return rc;
    cudaStream_t st = ctx->stream;
    Scratch sc(st);
    AngleGeom *geom;
    float2 *xpair, *xTpair;
    const size_t npair = (size_t)size * (size + 2);
    SYNK_CUDA(sc.reserve(Scratch::round(sizeof(AngleGeom) * (size_t)a) + 2 * Scratch::round(sizeof(float2) * npair) +
                         lists_bytes(a)),
              "cudaMallocAsync(scratch)");
    SYNK_CUDA(sc.get(&geom, (size_t)a), "cudaMallocAsync(geometry)");
    SYNK_CUDA(sc.get(&xpair, npair), "cudaMallocAsync(pair image)");
    SYNK_CUDA(sc.get(&xTpair, npair), "cudaMallocAsync(transposed pair image)");
    const ProbGeom P = make_geom(a, rhozero, deltarho, numrhos, size, geom);
    AngleLists L;
    SYNK_CUDA(make_setup(sc, angles, P, &L, st, image, xpair, xTpair), "setup kernel");
    SYNK_CUDA(launch_fp(P, L, xpair, xTpair, out, st), "forward projection kernel");
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
    cudaStream_t st = ctx->stream;
    Scratch sc(st);
    AngleGeom *geom;
    SYNK_CUDA(sc.reserve(Scratch::round(sizeof(AngleGeom) * (size_t)a) +
                         Scratch::round(sizeof(float) * 2 * (size_t)p) + lists_bytes(a)),
              "cudaMallocAsync(scratch)");
    SYNK_CUDA(sc.get(&geom, (size_t)a), "cudaMallocAsync(geometry)");
    const ProbGeom P = make_geom(a, rhozero, deltarho, numrhos, size_in, geom);
    AngleLists L;
    SYNK_CUDA(make_setup(sc, angles, P, &L, st), "setup kernel");
    float *scaled;   // scaled rows, or scaled detector pairs (launch_bp)
    SYNK_CUDA(sc.get(&scaled, 2 * (size_t)p), "cudaMallocAsync(scaled rows)");
    SYNK_CUDA(launch_bp(P, L, projections, out, st, scaled), "backprojection kernel");
    return SYNK_OK;
}

__global__ void fill_i32_kernel(int *p, int n, int v) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) p[i] = v;
}

int pick_fp_split(long long tasks, long long resident_warps, int size) {
    const int maxs = size / 16 > 8 ? 8 : (size / 16 < 1 ? 1 : size / 16);
    return pick_split(tasks, resident_warps, maxs);
}
int pick_bp_split(long long tasks, long long resident_warps, int64_t a) {
    const int maxs = a / 8 > 8 ? 8 : (a / 8 < 1 ? 1 : (int)(a / 8));
    return pick_split(tasks, resident_warps, maxs);
}

int valid_split(int s) { return s == 1 || s == 2 || s == 4 || s == 8; }

// `staging`: optional pinned host buffer of nprob SirtProblem entries; the
// problem table is uploaded from it (a copy a CUDA graph can capture) instead
// of from pageable memory.
// Engine choice by the work per iteration (FP ray-row steps + BP pixel-angle
// pairs), measured on GB300 with both engines forced on the same inputs:
// - up to kSmallWork the phase-split engine with the generic forward phase
//   (two launches per iteration, no grid barrier) beats the persistent kernel
//   1.08-1.32x (N=64-256, 1-64 slices);
// - above it, for one problem, the split engine whose forward phase runs on
//   the projector's own grid beats it 1.04-1.16x (N=256-1024, 1-256 slices;
//   N=2048 / 1 slice even); batches of several problems keep the persistent
//   kernel there.
constexpr double kSmallWork = 6.0e7;

int sirt_batch(synk_context *ctx, int nprob, const synk_sirt_problem *in, double tol, int grid_blocks,
               void *staging = nullptr) {
    int rc;
    if (nprob < 1 || nprob > (1 << 16)) return fail(ctx, SYNK_EINVAL, "bad problem count %d", nprob);
    if (!in) return fail(ctx, SYNK_EINVAL, "null problem table");
    if (!(tol >= 0.0) || !isfinite(tol)) return fail(ctx, SYNK_EINVAL, "tol must be finite and >= 0");
    if (grid_blocks < -1) return fail(ctx, SYNK_EINVAL, "grid_blocks must be -1, 0 or positive (got %d)", grid_blocks);
    cudaStream_t st = ctx->stream;
    int bps = 0;
    const int resident = sirt_persistent_grid(&bps);
    if (resident < 1) return fail(ctx, SYNK_ECUDA, "persistent SIRT kernel cannot be resident");
    int grid = resident;
    if (grid_blocks > 0 && grid_blocks < grid) grid = grid_blocks;
    const long long resident_warps = (long long)grid * 8;
    int max_iter = 0, max_slices = 1;
    bool any_work = false, want_res = false;
    for (int i = 0; i < nprob; ++i) {
        const synk_sirt_problem &q = in[i];
        if (!q.out || !q.angles || !q.projections) return fail(ctx, SYNK_EINVAL, "problem %d: null array pointer", i);
        if ((rc = check_geometry(ctx, q.a, q.rhozero, q.deltarho, q.numrhos, q.size))) return rc;
        if (q.nslices < 1 || q.nslices > (1 << 20)) return fail(ctx, SYNK_EINVAL, "problem %d: bad slice count %d", i, q.nslices);
        if (q.iterations < 0) return fail(ctx, SYNK_EINVAL, "iterations must be >= 0 (got %d)", q.iterations);
        if ((q.fp_split && !valid_split(q.fp_split)) || (q.bp_split && !valid_split(q.bp_split)))
            return fail(ctx, SYNK_EINVAL, "problem %d: work splits must be 0, 1, 2, 4 or 8", i);
        const size_t n = (size_t)q.size * q.size, pr = (size_t)q.a * q.numrhos;
        if ((double)q.nslices * (double)(n > pr ? n : pr) > 8.0e9)
            return fail(ctx, SYNK_EINVAL, "problem %d: slice stack too large", i);
        max_iter = q.iterations > max_iter ? q.iterations : max_iter;
        max_slices = q.nslices > max_slices ? q.nslices : max_slices;
        if (q.iterations > 0) any_work = true;
        if (q.residuals) want_res = true;
    }
    // Engine: one launch per phase and iteration (single problems, and small
    // batches), the fused persistent kernel otherwise (grid_blocks == -1
    // forces the split engine, > 0 the persistent kernel; 0 decides).
    double work = 0.0;   // FP ray-row steps + BP (pixel, angle) pairs per iteration
    for (int i = 0; i < nprob; ++i)
        work += (double)in[i].nslices * (double)in[i].a * in[i].size * ((double)in[i].size + in[i].numrhos);
    // (a captured plan keeps the persistent kernel unless forced: it cannot end the loop early)
    const bool split = grid_blocks == -1 || (grid_blocks == 0 && !staging && (nprob == 1 || work <= kSmallWork));
    int fpg = 0, bpg = 0;
    if (split && !sirt_phase_grids(&fpg, &bpg)) return fail(ctx, SYNK_ECUDA, "SIRT phase kernels cannot be resident");
    // one large problem: the split engine's forward phase on the projector's own grid
    const bool stack = split && nprob == 1 && work > kSmallWork && in[0].nslices <= 65535 &&
                       (in[0].a + 31) / 32 + 2 <= 65535;
    // the work splits fill the warps of the engine that runs the phases
    const long long fp_warps = split ? (long long)fpg * 8 : resident_warps;
    const long long bp_warps = split ? (long long)bpg * 8 : resident_warps;
    // start images
    for (int i = 0; i < nprob; ++i) {
        const synk_sirt_problem &q = in[i];
        const size_t bytes = sizeof(float) * (size_t)q.size * q.size * q.nslices;
        if (q.image) SYNK_CUDA(cudaMemcpyAsync(q.out, q.image, bytes, cudaMemcpyDeviceToDevice, st), "copy start");
        else SYNK_CUDA(cudaMemsetAsync(q.out, 0, bytes, st), "zero start");
    }
    if (!any_work && !want_res) {
        for (int i = 0; i < nprob; ++i)
            if (in[i].iterations_done)
                SYNK_CUDA(cudaMemsetAsync(in[i].iterations_done, 0, sizeof(int) * in[i].nslices, st), "memset");
        return SYNK_OK;
    }
    Scratch sc(st);
    std::vector<SirtProblem> host(nprob);
    for (int i = 0; i < nprob; ++i) {
        const synk_sirt_problem &q = in[i];
        SirtProblem &h = host[i];
        const size_t n = (size_t)q.size * q.size, pr = (size_t)q.a * q.numrhos;
        const size_t np = (size_t)q.size * (q.size + 2), K = (size_t)q.iterations + 1;
        AngleGeom *geom;
        float *R, *C, *xpad, *xTpad, *rr, *glen, *gcontrib;
        double *res2, *b2;
        int *stop_iter, *goff, *gcnt;
        int2 *graze, *graze_tmp;
        float *glen_tmp;
        // rays that only clip a corner pixel: per corner and angle at most
        // ceil(1/deltarho) + 1 (graze_list_kernel)
        const double gcapc = (double)q.a * (ceil(1.0 / (double)q.deltarho) + 1.0);
        const int graze_capc = (int)std::max(1.0, std::min({gcapc, (double)pr, (double)(1 << 26)}));
        SYNK_CUDA(sc.get(&geom, (size_t)q.a), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&graze, 4 * (size_t)graze_capc), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&glen, 4 * (size_t)graze_capc), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&gcontrib, 4 * (size_t)graze_capc * q.nslices), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&goff, 5), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&graze_tmp, 4 * (size_t)graze_capc), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&glen_tmp, 4 * (size_t)graze_capc), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&gcnt, 4), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&R, pr), "cudaMallocAsync(R)");
        SYNK_CUDA(sc.get(&C, n), "cudaMallocAsync(C)");
        SYNK_CUDA(sc.get(&xpad, np * q.nslices), "cudaMallocAsync(padded image)");
        SYNK_CUDA(sc.get(&xTpad, np * q.nslices), "cudaMallocAsync(padded transposed image)");
        SYNK_CUDA(sc.get(&rr, pr * q.nslices), "cudaMallocAsync(residual)");
        SYNK_CUDA(sc.get(&res2, K * q.nslices), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&b2, (size_t)q.nslices), "cudaMallocAsync");
        SYNK_CUDA(sc.get(&stop_iter, (size_t)q.nslices), "cudaMallocAsync");
        SYNK_CUDA(cudaMemsetAsync(res2, 0, sizeof(double) * K * q.nslices, st), "memset");
        SYNK_CUDA(cudaMemsetAsync(b2, 0, sizeof(double) * q.nslices, st), "memset");
        fill_i32_kernel<<<(unsigned)((q.nslices + 255) / 256), 256, 0, st>>>(stop_iter, q.nslices, INT_MAX);
        SYNK_CUDA(cudaGetLastError(), "fill kernel");
        h.P = make_geom(q.a, q.rhozero, q.deltarho, q.numrhos, q.size, geom);
        // the backprojection-grid backward phase (one large problem, every
        // window of its 64-row tiles in range) reads rr as detector pairs
        float *rrp = nullptr;
        if (stack && bp_windows_in_range(h.P, 64)) {
            SYNK_CUDA(sc.get(&rrp, 2 * pr * q.nslices), "cudaMallocAsync(residual pairs)");
            SYNK_CUDA(cudaMemsetAsync(rrp, 0, sizeof(float) * 2 * pr * q.nslices, st), "memset");
        }
        h.rrp = rrp;
        SYNK_CUDA(make_setup(sc, q.angles, h.P, &h.L, st), "setup kernel");
        SYNK_CUDA(launch_normalisers(h.P, R, C, graze, glen, goff, graze_tmp, glen_tmp, gcnt, graze_capc, st),
                  "normaliser kernels");
        // the listed rays' entries stay zero (their terms go to the corner pixels)
        SYNK_CUDA(cudaMemsetAsync(rr, 0, sizeof(float) * pr * q.nslices, st), "memset");
        SYNK_CUDA(launch_pad(q.out, xpad, xTpad, q.size, q.nslices, st), "pad kernel");
        SYNK_CUDA(launch_sumsq(q.projections, pr, q.nslices, b2, st), "norm kernel");
        h.R = R;
        h.graze = graze;
        h.glen = glen;
        h.gcontrib = gcontrib;
        h.goff = goff;
        h.graze_capc = graze_capc;
        h.C = C;
        h.b = q.projections;
        h.xpad = xpad;
        h.xTpad = xTpad;
        h.rr = rr;
        h.res2 = res2;
        h.b2 = b2;
        h.stop_iter = stop_iter;
        h.residuals = q.residuals;
        h.iters_done = q.iterations_done;
        h.nslices = q.nslices;
        h.iterations = q.iterations;
        // warp tasks per phase: one detector x 32 angles (FP), one 32-column x 4-row strip (BP)
        const long long fp_tasks = (long long)q.nslices * q.numrhos * ((q.a + 31) / 32);
        const long long bp_tasks = (long long)q.nslices * ((q.size + 3) / 4) * ((q.size + 31) / 32);
        const long long fp_share = nprob > 1 ? fp_warps / nprob + 1 : fp_warps;
        const long long bp_share = nprob > 1 ? bp_warps / nprob + 1 : bp_warps;
        h.bp_inrange = bp_windows_in_range(h.P, 32) ? 1 : 0;   // BP tiles of bp_pix*(8/bp_split) <= 32 rows
        h.fp_split = q.fp_split ? q.fp_split : pick_fp_split(fp_tasks, fp_share, q.size);
        h.bp_split = q.bp_split ? q.bp_split : pick_bp_split(bp_tasks, bp_share, q.a);
        // The phase kernels' items are blocks of 8 warps.  Measured with the
        // split engine at N=64/128/256 (1 slice, 200 iterations), its forward
        // phase is fastest with the rays' rows split as far as keeps the warps
        // within the resident ones (S = 8/8/2 there, parts of >= 8 rows), and
        // the backward phase with the fewest pixels per thread (1 of 4) that
        // still give 3/4 of the resident blocks an item: N=128 5.88 -> 4.69 ms,
        // N=64 4.25 -> 3.44 ms (before the chained launches).
        if (split && !stack && !q.fp_split) {
            const int maxs = q.size / 8 > 8 ? 8 : (q.size / 8 < 1 ? 1 : q.size / 8);
            int S = 1;
            while (S < maxs && fp_tasks * S * 2 <= fp_share) S *= 2;
            h.fp_split = S;
        }
        h.bp_pix = 4;
        const long long tiles_x = (q.size + 31) / 32;
        const long long bp_blocks = (split ? bpg : grid) / (nprob > 1 ? nprob : 1) + 1;
        while (h.bp_pix > 1) {
            const int TR = h.bp_pix * (8 / h.bp_split);
            const long long items = (long long)q.nslices * tiles_x * ((q.size + TR - 1) / TR);
            if (items * 4 >= bp_blocks * 3) break;
            h.bp_pix >>= 1;
        }
        h.fp_ips = h.bp_ips = 0;
        h.fp_begin = h.bp_begin = 0;
    }
    // largest problems first: with the atomic hand-out the long items start early
    std::vector<int> order(nprob);
    for (int i = 0; i < nprob; ++i) order[i] = i;
    std::stable_sort(order.begin(), order.end(), [&](int x, int y) {
        const double cx = (double)in[x].size * in[x].size * in[x].a * in[x].nslices;
        const double cy = (double)in[y].size * in[y].size * in[y].a * in[y].nslices;
        return cx > cy;
    });
    std::vector<SirtProblem> sorted(nprob);
    for (int i = 0; i < nprob; ++i) sorted[i] = host[order[i]];
    SirtProblem *dprobs;
    long long *totals;
    unsigned *words;
    SYNK_CUDA(sc.get(&dprobs, (size_t)nprob), "cudaMallocAsync(problem table)");
    SYNK_CUDA(sc.get(&totals, 2), "cudaMallocAsync");
    SYNK_CUDA(sc.get(&words, 8), "cudaMallocAsync");
    if (staging) {
        // pinned copy: stays valid for every replay of a captured graph
        memcpy(staging, sorted.data(), sizeof(SirtProblem) * nprob);
        SYNK_CUDA(cudaMemcpyAsync(dprobs, staging, sizeof(SirtProblem) * nprob, cudaMemcpyHostToDevice, st),
                  "upload problem table");
    } else {
        // from pageable memory: the copy is staged before the call returns, so
        // the host vector may go out of scope afterwards
        SYNK_CUDA(cudaMemcpyAsync(dprobs, sorted.data(), sizeof(SirtProblem) * nprob, cudaMemcpyHostToDevice, st),
                  "upload problem table");
    }
    SYNK_CUDA(cudaMemsetAsync(words, 0, sizeof(unsigned) * 8, st), "memset");
    SYNK_CUDA(launch_sirt_plan(dprobs, nprob, totals, st), "plan kernel");
    SirtParams sp;
    sp.probs = dprobs;
    sp.totals = totals;
    sp.nprob = nprob;
    sp.max_iterations = max_iter;
    sp.bar = words;
    sp.work = words + 4;
    sp.status = ctx->d_status;
    sp.timeout_ns = ctx->barrier_timeout_ns;
    sp.barrier_extra = ctx->barrier_extra;
    sp.tol2 = tol > 0.0 ? tol * tol : 0.0;
    sp.record_final = want_res ? 1 : 0;
    sp.dynamic = nprob > 1 ? 1 : 0;
    if (split) {
        sp.dynamic = 0;
        int *active = reinterpret_cast<int *>(words + 7);
        // the early exit reads the active count on the host: not inside a graph
        // capture (the library's own plan, or a caller capturing this stream)
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cap) != cudaSuccess) cap = cudaStreamCaptureStatusNone;
        const bool can_poll = sp.tol2 > 0.0 && !staging && cap == cudaStreamCaptureStatusNone;
        int poll_slot = 0, poll_prev = -1;
        for (int it = 0; it <= max_iter; ++it) {
            if (stack) SYNK_CUDA(launch_sirt_fp_stack(host[0], it, sp.tol2, sp.record_final, st), "SIRT forward phase");
            else SYNK_CUDA(launch_sirt_fp_phase(sp, it, fpg, st), "SIRT forward phase");
            if (it == max_iter) break;
            if (host[0].rrp) SYNK_CUDA(launch_sirt_bp_stack(host[0], it, sp.tol2, active, st), "SIRT backward phase");
            else SYNK_CUDA(launch_sirt_bp_phase(sp, it, active, bpg, st), "SIRT backward phase");
            // Every 16 iterations the count of slices still updating is copied
            // to pinned memory behind the backward phase, and the host waits
            // for the copy queued 16 iterations earlier, not for the stream:
            // the GPU keeps the iterations in between queued (the chained
            // launches stay chained) and the loop ends once no slice updates
            // any more.  The at most 16-31 iterations already queued then skip
            // their work in the kernels (stopping rule per slice).  Draining
            // the stream at each check cost more than stopping saved (N=128:
            // 184 iterations to the residual 4.20 ms, 200 iterations 3.96 ms).
            if (can_poll && (it & 15) == 15) {
                SYNK_CUDA(cudaMemcpyAsync(ctx->h_poll + poll_slot, active, sizeof(int), cudaMemcpyDeviceToHost, st),
                          "read active");
                SYNK_CUDA(cudaEventRecord(ctx->poll_ev[poll_slot], st), "record poll");
                if (poll_prev >= 0) {
                    SYNK_CUDA(cudaEventSynchronize(ctx->poll_ev[poll_prev]), "wait poll");
                    if (ctx->h_poll[poll_prev] == 0) break;
                }
                poll_prev = poll_slot;
                poll_slot ^= 1;
            }
        }
    } else {
        SYNK_CUDA(launch_sirt_persistent(sp, grid, st), "persistent SIRT kernel");
    }
    for (int i = 0; i < nprob; ++i)
        SYNK_CUDA(launch_unpad(host[i].xpad, in[i].out, in[i].size, in[i].nslices, st), "unpad kernel");
    SYNK_CUDA(launch_sirt_finalize(dprobs, nprob, max_slices, sp.record_final, st), "finalize kernel");
    return SYNK_OK;
}

int sirt_slices(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero, float deltarho,
                int64_t numrhos, int64_t size, int64_t nslices, const float *image, const float *projections,
                int32_t iterations, const synk_sirt_options *opts) {
    synk_sirt_problem q = {};
    q.angles = angles;
    q.a = a;
    q.rhozero = rhozero;
    q.deltarho = deltarho;
    q.numrhos = (int32_t)numrhos;
    q.size = (int32_t)size;
    q.nslices = (int32_t)nslices;
    q.iterations = iterations;
    q.image = image;
    q.projections = projections;
    q.out = out;
    q.residuals = opts ? opts->residuals : nullptr;
    q.iterations_done = opts ? opts->iterations_done : nullptr;
    q.fp_split = opts ? opts->fp_split : 0;
    q.bp_split = opts ? opts->bp_split : 0;
    if (numrhos > INT32_MAX || size > INT32_MAX || nslices > INT32_MAX) return fail(ctx, SYNK_EINVAL, "size out of range");
    return sirt_batch(ctx, 1, &q, opts ? opts->tol : 0.0, opts ? opts->grid_blocks : 0);
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
    // Keep freed stream-ordered scratch in the device's default pool instead of
    // returning it to the driver at every synchronisation (the default release
    // threshold 0 makes each call re-map its scratch).
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
        uint64_t keep = ~0ull;
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    synk_context *ctx = new synk_context();
    ctx->device = device;
    ctx->stream = static_cast<cudaStream_t>(stream);
    if (cudaMalloc(&ctx->d_status, sizeof(int)) != cudaSuccess ||
        cudaMemset(ctx->d_status, 0, sizeof(int)) != cudaSuccess ||
        cudaHostAlloc(&ctx->h_poll, 2 * sizeof(int), cudaHostAllocDefault) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->poll_ev[0], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&ctx->poll_ev[1], cudaEventDisableTiming) != cudaSuccess) {
        synk_context_free(ctx);
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
    if (ctx->h_poll) cudaFreeHost(ctx->h_poll);
    for (cudaEvent_t e : ctx->poll_ev)
        if (e) cudaEventDestroy(e);
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

int synk_context_set_barrier_limit(synk_context *ctx, uint64_t timeout_ns, int32_t missing_blocks) {
    if (!ctx) return SYNK_EINVAL;
    ctx->err.clear();
    if (timeout_ns < 1000ull || timeout_ns > 60000000000ull)
        return fail(ctx, SYNK_EINVAL, "barrier time limit must be in [1 us, 60 s] (got %llu ns)",
                    (unsigned long long)timeout_ns);
    if (missing_blocks < 0 || missing_blocks > 1024)
        return fail(ctx, SYNK_EINVAL, "missing_blocks must be in [0, 1024] (got %d)", missing_blocks);
    ctx->barrier_timeout_ns = timeout_ns;
    ctx->barrier_extra = (unsigned)missing_blocks;
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

int synk_sirt_resident_blocks(void) { return sirt_persistent_grid(nullptr); }

struct synk_sirt_plan {
    int device = 0;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    void *staging = nullptr;
};

static void plan_release(synk_sirt_plan *p) {
    if (!p) return;
    if (p->exec) cudaGraphExecDestroy(p->exec);
    if (p->graph) cudaGraphDestroy(p->graph);
    if (p->staging) cudaFreeHost(p->staging);
    delete p;
}

int synk_sirt_plan_new(synk_context *ctx, synk_sirt_plan **out, int32_t nprob, const synk_sirt_problem *probs,
                       double tol, int32_t grid_blocks) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out) return fail(ctx, SYNK_EINVAL, "null pointer");
    *out = nullptr;
    if (nprob < 1 || nprob > (1 << 16) || !probs) return fail(ctx, SYNK_EINVAL, "bad problem table");
    synk_sirt_plan *plan = new synk_sirt_plan();
    plan->device = ctx->device;
    cudaError_t e = cudaHostAlloc(&plan->staging, sizeof(SirtProblem) * (size_t)nprob, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        plan_release(plan);
        return cuda_fail(ctx, e, "cudaHostAlloc(problem table)");
    }
    cudaStream_t cs;
    if ((e = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking)) != cudaSuccess) {
        plan_release(plan);
        return cuda_fail(ctx, e, "cudaStreamCreate");
    }
    cudaStream_t saved = ctx->stream;
    ctx->stream = cs;
    e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) rc = sirt_batch(ctx, nprob, probs, tol, grid_blocks, plan->staging);
    cudaGraph_t g = nullptr;
    const cudaError_t e2 = e == cudaSuccess ? cudaStreamEndCapture(cs, &g) : e;
    ctx->stream = saved;
    cudaStreamDestroy(cs);
    if (e != cudaSuccess || e2 != cudaSuccess || rc != SYNK_OK) {
        if (g) cudaGraphDestroy(g);
        plan_release(plan);
        if (rc != SYNK_OK) return rc;
        return cuda_fail(ctx, e != cudaSuccess ? e : e2, "stream capture of the SIRT solve");
    }
    plan->graph = g;
    if ((e = cudaGraphInstantiate(&plan->exec, g, 0)) != cudaSuccess) {
        plan_release(plan);
        return cuda_fail(ctx, e, "cudaGraphInstantiate");
    }
    *out = plan;
    return SYNK_OK;
}

int synk_sirt_plan_launch(synk_context *ctx, synk_sirt_plan *plan) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!plan || !plan->exec) return fail(ctx, SYNK_EINVAL, "null plan");
    SYNK_CUDA(cudaGraphLaunch(plan->exec, ctx->stream), "cudaGraphLaunch");
    return SYNK_OK;
}

void synk_sirt_plan_free(synk_sirt_plan *plan) {
    if (!plan) return;
    cudaSetDevice(plan->device);
    cudaDeviceSynchronize();
    plan_release(plan);
}

int synk_sirt_batch(synk_context *ctx, int32_t nprob, const synk_sirt_problem *probs, double tol,
                    int32_t grid_blocks) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    return sirt_batch(ctx, nprob, probs, tol, grid_blocks);
}

int synk_sirt_slices(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                     float deltarho, int32_t numrhos, int32_t size, int32_t nslices, const float *image,
                     const float *projections, int32_t iterations, const synk_sirt_options *opts) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    return sirt_slices(ctx, out, angles, a, rhozero, deltarho, numrhos, size, nslices, image, projections,
                       iterations, opts);
}

static void csr_release(synk_csr *m) {
    if (!m) return;
    cudaFree(m->ptr); cudaFree(m->ptr_t);
    cudaFree(m->idx); cudaFree(m->idx_t);
    cudaFree(m->vals); cudaFree(m->vals_t);
    delete m;
}

int synk_gemm_bf16(synk_context *ctx, const uint16_t *A, const uint16_t *B, float *C, int32_t M, int32_t N,
                   int32_t K) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!A || !B || !C) return fail(ctx, SYNK_EINVAL, "null pointer");
    if (M <= 0 || M % 128 || N < 16 || N > 256 || N % 16 || K <= 0 || K % 64)
        return fail(ctx, SYNK_EINVAL, "gemm shape M=%d N=%d K=%d not supported", M, N, K);
    SYNK_CUDA(unet::gemm_bf16(A, B, C, M, N, K, ctx->d_status, ctx->barrier_timeout_ns, ctx->stream), "tcgen05 gemm");
    return SYNK_OK;
}

int synk_conv3x3_bf16(synk_context *ctx, const uint16_t *x, int32_t ldx, int32_t xoff, int32_t Cin, int32_t B,
                      int32_t H, int32_t W, const uint16_t *w, const float *bias, uint16_t *y, int32_t ldy,
                      int32_t yoff, int32_t Cout, int32_t epi, const uint16_t *mask, int32_t ldm, int32_t moff) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!x || !w || !y) return fail(ctx, SYNK_EINVAL, "null pointer");
    if ((epi == unet::EPI_BIAS_RELU || epi == unet::EPI_BIAS) && !bias) return fail(ctx, SYNK_EINVAL, "null bias");
    if (epi == unet::EPI_MASK && !mask) return fail(ctx, SYNK_EINVAL, "null mask");
    if (B <= 0 || H <= 0 || W <= 0) return fail(ctx, SYNK_EINVAL, "bad image shape");
    unet::ConvArgs c = {x, ldx, xoff, Cin, B, H, W, w, bias, y, ldy, yoff, Cout, mask, ldm, moff};
    cudaError_t e = unet::conv3x3(c, epi, ctx->d_status, ctx->barrier_timeout_ns, ctx->stream);
    if (e == cudaErrorInvalidValue) return fail(ctx, SYNK_EINVAL, "conv3x3 shape not supported (Cin=%d Cout=%d H=%d W=%d)", Cin, Cout, H, W);
    SYNK_CUDA(e, "tcgen05 conv3x3");
    return SYNK_OK;
}

int synk_conv3x3_wgrad_bf16(synk_context *ctx, const uint16_t *dyT, const uint16_t *xT3, float *dw, int32_t Cin,
                            int32_t Cout, int32_t B, int32_t H, int32_t W, int32_t ksplit) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!dyT || !xT3 || !dw) return fail(ctx, SYNK_EINVAL, "null pointer");
    if (B <= 0 || H <= 0 || W <= 0 || ksplit < 1) return fail(ctx, SYNK_EINVAL, "bad shape");
    unet::WgradArgs a = {dyT, xT3, dw, Cin, Cout, B, H, W, ksplit};
    cudaError_t e = unet::conv3x3_wgrad(a, ctx->d_status, ctx->barrier_timeout_ns, ctx->stream);
    if (e == cudaErrorInvalidValue) return fail(ctx, SYNK_EINVAL, "wgrad shape not supported");
    SYNK_CUDA(e, "tcgen05 wgrad");
    return SYNK_OK;
}

struct synk_unet {
    int device = 0;
    int size = 0, max_batch = 0;
    unet::Net *net = nullptr;
};

int synk_unet_new(synk_context *ctx, synk_unet **out, int32_t max_batch, int32_t size, uint64_t seed) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out) return fail(ctx, SYNK_EINVAL, "null pointer");
    *out = nullptr;
    if (size < 256 || size % 256 || size > 4096) return fail(ctx, SYNK_EINVAL, "U-Net size must be a multiple of 256 (got %d)", size);
    if (max_batch < 1 || max_batch > 1024) return fail(ctx, SYNK_EINVAL, "bad batch %d", max_batch);
    unet::Net *n = nullptr;
    SYNK_CUDA(unet::net_create(&n, max_batch, size, seed, ctx->stream), "U-Net allocation");
    synk_unet *h = new synk_unet();
    h->device = ctx->device;
    h->size = size;
    h->max_batch = max_batch;
    h->net = n;
    *out = h;
    return SYNK_OK;
}

void synk_unet_free(synk_unet *net) {
    if (!net) return;
    cudaSetDevice(net->device);
    cudaDeviceSynchronize();
    unet::net_free(net->net);
    delete net;
}

int64_t synk_unet_num_params(const synk_unet *net) { return net ? unet::net_nparams(net->net) : 0; }

int synk_unet_params(synk_context *ctx, synk_unet *net, float *dst, int32_t direction) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!net || !dst) return fail(ctx, SYNK_EINVAL, "null pointer");
    const size_t bytes = sizeof(float) * (size_t)unet::net_nparams(net->net);
    if (direction == 0) {
        SYNK_CUDA(cudaMemcpyAsync(dst, unet::net_params(net->net), bytes, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
    } else {
        SYNK_CUDA(cudaMemcpyAsync(unet::net_params(net->net), dst, bytes, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        SYNK_CUDA(unet::net_refresh_weights(net->net, ctx->stream), "weight copies");
    }
    return SYNK_OK;
}

int synk_unet_optimizer_state(synk_context *ctx, synk_unet *net, float *m, float *v, int64_t *step,
                              int32_t direction) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!net || !m || !v || !step) return fail(ctx, SYNK_EINVAL, "null pointer");
    if (direction != 0 && direction != 1) return fail(ctx, SYNK_EINVAL, "direction must be 0 or 1 (got %d)", direction);
    const size_t bytes = sizeof(float) * (size_t)unet::net_nparams(net->net);
    int *st = unet::net_adam_step(net->net);
    if (direction == 0) {
        SYNK_CUDA(cudaMemcpyAsync(m, unet::net_adam_m(net->net), bytes, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        SYNK_CUDA(cudaMemcpyAsync(v, unet::net_adam_v(net->net), bytes, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        *step = *st;
    } else {
        if (*step < 0 || *step > INT32_MAX) return fail(ctx, SYNK_EINVAL, "Adam step %lld out of range", (long long)*step);
        SYNK_CUDA(cudaMemcpyAsync(unet::net_adam_m(net->net), m, bytes, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        SYNK_CUDA(cudaMemcpyAsync(unet::net_adam_v(net->net), v, bytes, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
        *st = (int)*step;
    }
    return SYNK_OK;
}

int synk_unet_forward(synk_context *ctx, synk_unet *net, const float *x, float *y, int32_t batch) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!net || !x || !y) return fail(ctx, SYNK_EINVAL, "null pointer");
    if (batch < 1 || batch > net->max_batch) return fail(ctx, SYNK_EINVAL, "batch %d outside [1, %d]", batch, net->max_batch);
    SYNK_CUDA(unet::net_forward(net->net, batch, x, y, nullptr, ctx->d_status, ctx->barrier_timeout_ns, ctx->stream),
              "U-Net forward");
    return SYNK_OK;
}

int synk_unet_train_step(synk_context *ctx, synk_unet *net, const float *x, const float *target, int32_t batch,
                         float lr, int32_t apply, double *loss) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!net || !x || !target) return fail(ctx, SYNK_EINVAL, "null pointer");
    if (batch < 1 || batch > net->max_batch) return fail(ctx, SYNK_EINVAL, "batch %d outside [1, %d]", batch, net->max_batch);
    if (!(lr >= 0.0f) || !isfinite(lr)) return fail(ctx, SYNK_EINVAL, "bad learning rate");
    unet::Net *n = net->net;
    cudaStream_t st = ctx->stream;
    SYNK_CUDA(cudaMemsetAsync(unet::net_grads(n), 0, sizeof(float) * (size_t)unet::net_nparams(n), st), "zero grads");
    SYNK_CUDA(unet::net_forward(n, batch, x, nullptr, target, ctx->d_status, ctx->barrier_timeout_ns, st), "U-Net forward");
    SYNK_CUDA(unet::net_backward(n, batch, ctx->d_status, ctx->barrier_timeout_ns, st), "U-Net backward");
    if (loss) SYNK_CUDA(cudaMemcpyAsync(loss, unet::net_loss(n), sizeof(double), cudaMemcpyDeviceToDevice, st), "loss");
    if (apply) SYNK_CUDA(unet::net_adam(n, lr, st), "Adam");
    return SYNK_OK;
}

int synk_unet_gradients(synk_context *ctx, synk_unet *net, float *dst) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!net || !dst) return fail(ctx, SYNK_EINVAL, "null pointer");
    const size_t bytes = sizeof(float) * (size_t)unet::net_nparams(net->net);
    SYNK_CUDA(cudaMemcpyAsync(dst, unet::net_grads(net->net), bytes, cudaMemcpyDeviceToDevice, ctx->stream), "copy");
    return SYNK_OK;
}

int synk_csr_new(synk_context *ctx, synk_csr **out, const float *angles, int64_t a, float rhozero, float deltarho,
                 int32_t numrhos, int32_t size) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out || !angles) return fail(ctx, SYNK_EINVAL, "null pointer");
    *out = nullptr;
    if ((rc = check_geometry(ctx, a, rhozero, deltarho, numrhos, size))) return rc;
    const int64_t rows = a * (int64_t)numrhos, cols = (int64_t)size * size;
    if (rows >= (1ll << 31) || cols >= (1ll << 31))
        return fail(ctx, SYNK_EINVAL, "matrix dimensions exceed int32 indices");
    cudaStream_t st = ctx->stream;
    synk_csr *m = new synk_csr();
    m->device = ctx->device;
    m->rows = rows;
    m->cols = cols;
    Scratch sc(st);
    AngleGeom *geom;
    int *counts;
    int64_t *sums, *total;
    const int64_t maxn = rows > cols ? rows : cols;
    cudaError_t e;
#define CSR_TRY(call, what)                         \
    do {                                            \
        e = (call);                                 \
        if (e != cudaSuccess) {                     \
            csr_release(m);                         \
            return cuda_fail(ctx, e, what);         \
        }                                           \
    } while (0)
    CSR_TRY(sc.get(&geom, (size_t)a), "cudaMallocAsync");
    CSR_TRY(sc.get(&counts, (size_t)maxn), "cudaMallocAsync");
    CSR_TRY(sc.get(&sums, (size_t)(maxn / 1024 + 2)), "cudaMallocAsync");
    CSR_TRY(sc.get(&total, 2), "cudaMallocAsync");
    CSR_TRY(launch_geometry(angles, (int)a, geom, st), "geometry kernel");
    const ProbGeom P = make_geom(a, rhozero, deltarho, numrhos, size, geom);
    for (int tr = 0; tr < 2; ++tr) {
        const int64_t n = tr ? cols : rows;
        int64_t **pp = tr ? &m->ptr_t : &m->ptr;
        int **ip = tr ? &m->idx_t : &m->idx;
        float **vp = tr ? &m->vals_t : &m->vals;
        CSR_TRY(cudaMalloc(pp, sizeof(int64_t) * (n + 1)), "cudaMalloc(row pointers)");
        CSR_TRY(launch_csr_count(P, tr != 0, counts, st), "count kernel");
        CSR_TRY(exclusive_scan(counts, n, *pp, sums, total, st), "scan kernels");
        int64_t nnz = 0;
        CSR_TRY(cudaMemcpyAsync(&nnz, total, sizeof nnz, cudaMemcpyDeviceToHost, st), "read nnz");
        CSR_TRY(cudaStreamSynchronize(st), "cudaStreamSynchronize");
        if (tr && nnz != m->nnz) {
            csr_release(m);
            return fail(ctx, SYNK_ECUDA, "transpose has %lld non-zeros, A has %lld", (long long)nnz, (long long)m->nnz);
        }
        m->nnz = nnz;
        CSR_TRY(cudaMalloc(ip, sizeof(int) * (nnz + 1)), "cudaMalloc(indices)");
        CSR_TRY(cudaMalloc(vp, sizeof(float) * (nnz + 1)), "cudaMalloc(values)");
        CSR_TRY(launch_csr_fill(P, tr != 0, *pp, *ip, *vp, st), "fill kernel");
    }
#undef CSR_TRY
    *out = m;
    return SYNK_OK;
}

void synk_csr_free(synk_csr *m) {
    if (!m) return;
    cudaSetDevice(m->device);
    cudaDeviceSynchronize();
    csr_release(m);
}

int synk_csr_shape(const synk_csr *m, int64_t *rows, int64_t *cols, int64_t *nnz) {
    if (!m) return SYNK_EINVAL;
    if (rows) *rows = m->rows;
    if (cols) *cols = m->cols;
    if (nnz) *nnz = m->nnz;
    return SYNK_OK;
}

int synk_csr_arrays(const synk_csr *m, int transpose, const int64_t **rowptr, const int32_t **colidx,
                    const float **vals) {
    if (!m) return SYNK_EINVAL;
    if (rowptr) *rowptr = transpose ? m->ptr_t : m->ptr;
    if (colidx) *colidx = transpose ? m->idx_t : m->idx;
    if (vals) *vals = transpose ? m->vals_t : m->vals;
    return SYNK_OK;
}

int synk_csr_spmv(synk_context *ctx, const synk_csr *m, const float *x, float *y) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!m || !x || !y) return fail(ctx, SYNK_EINVAL, "null pointer");
    SYNK_CUDA(launch_spmv(m->rows, m->ptr, nullptr, m->idx, m->vals, x, y, ctx->stream), "spmv kernel");
    return SYNK_OK;
}

int synk_csr_spmv_t(synk_context *ctx, const synk_csr *m, const float *y, float *x) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!m || !x || !y) return fail(ctx, SYNK_EINVAL, "null pointer");
    SYNK_CUDA(launch_spmv(m->cols, m->ptr_t, nullptr, m->idx_t, m->vals_t, y, x, ctx->stream), "spmv kernel");
    return SYNK_OK;
}

int synk_spmv_csr32(synk_context *ctx, int64_t rows, const int32_t *rowptr, const int32_t *colidx,
                    const float *vals, const float *x, float *y) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (rows < 0) return fail(ctx, SYNK_EINVAL, "negative row count");
    if (rows == 0) return SYNK_OK;
    if (!rowptr || !colidx || !vals || !x || !y) return fail(ctx, SYNK_EINVAL, "null pointer");
    SYNK_CUDA(launch_spmv(rows, nullptr, rowptr, colidx, vals, x, y, ctx->stream), "spmv kernel");
    return SYNK_OK;
}

int synk_compare(synk_context *ctx, synk_compare_result *out, const float *sane, const float *test, int64_t n,
                 float tol) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (n < 0) return fail(ctx, SYNK_EINVAL, "negative length");
    if (!out || (n && (!sane || !test))) return fail(ctx, SYNK_EINVAL, "null pointer");
    SYNK_CUDA(launch_compare(sane, test, n, tol, out, ctx->stream), "compare kernel");
    return SYNK_OK;
}

}  // extern "C"

namespace {

// tools/diff.fut, mse.fut and sanityCheck.fut share std_dev = 0.05f32.
constexpr float kToolsStdDev = 0.05f;

int compare_program(synk_context *ctx, int what, void *out, const float *sane, const float *test, int64_t n) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (n < 0) return fail(ctx, SYNK_EINVAL, "negative length");
    if (!out || (n && (!sane || !test))) return fail(ctx, SYNK_EINVAL, "null pointer");
    Scratch scr(ctx->stream);
    CompareResult *r = nullptr;
    SYNK_CUDA(scr.get(&r, 1), "scratch");
    SYNK_CUDA(launch_compare(sane, test, n, kToolsStdDev, r, ctx->stream), "compare kernel");
    SYNK_CUDA(launch_compare_finish(r, n, what, out, ctx->stream), "compare kernel");
    return SYNK_OK;
}

}  // namespace

extern "C" {

int synk_diff(synk_context *ctx, int32_t *out, const float *sane, const float *test, int64_t n) {
    return compare_program(ctx, 0, out, sane, test, n);
}

int synk_mse(synk_context *ctx, float *out, const float *sane, const float *test, int64_t n) {
    return compare_program(ctx, 1, out, sane, test, n);
}

int synk_sanityCheck(synk_context *ctx, uint8_t *out, const float *sane, const float *test, int64_t n) {
    return compare_program(ctx, 2, out, sane, test, n);
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Backprojection without any allocation.
//
// Some callers of this library cannot let it allocate device memory: programs
// that reserve all free device memory for their own allocator at start-up (a
// library cudaMalloc/cudaMallocAsync then fails or fragments their pool), and
// acquisition loops that must never enter the CUDA allocator while frames are
// streaming, because an allocation can take the driver's allocator lock or
// synchronise the device and stall a running stream.
//
// synk_backprojection_noalloc is synk_backprojection with its scratch (the
// per-angle geometry table and the angle lists) kept in one file-scope
// __device__ array instead of stream-ordered allocations.  The array is sized
// for at most SYNK_NOALLOC_MAX_ANGLES angles (about 448 KiB) and every GPU on
// which the library is loaded holds it until the process exits.  Every call
// shares the array and overwrites it completely before reading it (nothing in
// it has to start at zero), so calls that overlap on the GPU -- on two streams,
// or from two host threads -- race on it and must be serialised by the caller.
// ---------------------------------------------------------------------------

namespace {

struct NoAllocScratch {
    AngleGeom geom[SYNK_NOALLOC_MAX_ANGLES];
    int order[SYNK_NOALLOC_MAX_ANGLES + 64];
    int exact[SYNK_NOALLOC_MAX_ANGLES];
    int counts[4];
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

constexpr int kMaxDevices = 256;
std::mutex g_noalloc_mutex;
void *g_noalloc_addr[kMaxDevices] = {};

// Device address of the scratch array on the current device (set-up once per
// device; the host-side symbol itself is not a device address).
int noalloc_scratch(synk_context *ctx, NoAllocScratch **out) {
    if (ctx->device < 0 || ctx->device >= kMaxDevices) return fail(ctx, SYNK_EINVAL, "device index out of range");
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (!g_noalloc_addr[ctx->device]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) return cuda_fail(ctx, e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                                                     "cudaGetSymbolAddress(no-allocation scratch)");
        g_noalloc_addr[ctx->device] = p;
    }
    *out = static_cast<NoAllocScratch *>(g_noalloc_addr[ctx->device]);
    return SYNK_OK;
}

}  // namespace

extern "C" int synk_backprojection_noalloc(synk_context *ctx, float *out, const float *angles, int64_t a,
                                           float rhozero, float deltarho, int32_t size, const float *projections,
                                           int64_t p) {
    int rc = check_ctx(ctx);   // makes the context's device current
    if (rc) return rc;
    if (!out || !angles || !projections) return fail(ctx, SYNK_EINVAL, "null array pointer");
    if (a < 1) return fail(ctx, SYNK_EINVAL, "need at least one angle (got %lld)", (long long)a);
    if (a > SYNK_NOALLOC_MAX_ANGLES)
        return fail(ctx, SYNK_EINVAL, "synk_backprojection_noalloc supports at most %d angles (got %lld); "
                    "use synk_backprojection", SYNK_NOALLOC_MAX_ANGLES, (long long)a);
    if (p < a || p % a) return fail(ctx, SYNK_EINVAL, "projection length %lld is not a multiple of %lld angles",
                                    (long long)p, (long long)a);
    const int64_t numrhos = p / a;
    if ((rc = check_geometry(ctx, a, rhozero, deltarho, numrhos, size))) return rc;
    NoAllocScratch *sc = nullptr;
    if ((rc = noalloc_scratch(ctx, &sc))) return rc;
    cudaStream_t st = ctx->stream;
    SYNK_CUDA(launch_geometry(angles, (int)a, sc->geom, st), "geometry kernel");
    const ProbGeom P = make_geom(a, rhozero, deltarho, numrhos, size, sc->geom);
    SYNK_CUDA(launch_angle_lists(P, sc->order, sc->exact, sc->counts, st), "angle lists kernel");
    AngleLists L;
    L.order = sc->order;
    L.exact = sc->exact;
    L.counts = sc->counts;
    SYNK_CUDA(launch_bp(P, L, projections, out, st, nullptr), "backprojection kernel");
    return SYNK_OK;
}

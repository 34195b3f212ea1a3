/*
 * libsynk: GB300-native (sm_103a) parallel-beam projection and SIRT.
 *
 * C ABI of the drop-in boundary.  The reference (tomograph/synkrotomo) is a
 * set of Futhark programs whose entry point `main` is exposed by Futhark's
 * generated libraries: `futhark pyopencl --library` (Makefile:1-4, the Python
 * classes of README.md:21-25) and `futhark c --library` (Makefile:6-9), whose
 * C API is a context object (futhark_context_new / _sync / _get_error /
 * _free) plus one `futhark_entry_main(ctx, &out, in0, in1, ...)` per program.
 * This header keeps that shape: one context per device and stream, one entry
 * point per reference program with the program's own argument order, the
 * output first, an int status (0 = success), errors described by
 * synk_context_get_error().
 *
 * Conventions:
 *  - Every array argument is a DEVICE pointer to contiguous float32 data of
 *    the stated length; lengths are element counts.  Scalars follow the
 *    reference's f32 / i32 types.
 *  - Entry points are stream-ordered: they enqueue work on the context's
 *    stream and return launch/validation errors.  Errors that happen while
 *    the GPU runs (a persistent kernel's grid barrier that timed out) are
 *    reported by the next synk_context_sync().
 *  - Inputs are never modified.  Scratch memory is taken from CUDA's
 *    stream-ordered allocator (cudaMallocAsync) on the context's stream.
 *  - A context is used by one host thread at a time.
 *  - Geometry: ray (angle theta, detector r) is the line
 *    rho = x*cos(theta) - y*sin(theta), rho = rhozero + r*deltarho,
 *    x = col - size/2, y = row - size/2 (futhark/forwardprojection.fut:26-29).
 *    Images are row-major [size*size]; sinograms angle-major [a*numrhos].
 */
#ifndef SYNK_H
#define SYNK_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define SYNK_OK 0
#define SYNK_EINVAL 1    /* bad argument (shape, size, null pointer)       */
#define SYNK_ECUDA 2     /* a CUDA runtime call failed                     */
#define SYNK_ETIMEOUT 3  /* a persistent kernel's grid barrier timed out   */
#define SYNK_ENOMEM 4    /* device allocation failed                       */

typedef struct synk_context synk_context;

/* ---- context (futhark_context_new / _free / _sync / _get_error) ---- */

/* Creates a context on CUDA device `device` that enqueues on `stream`
 * (a cudaStream_t; NULL = the legacy default stream). */
int synk_context_new(synk_context **out, int device, void *stream);
void synk_context_free(synk_context *ctx);
/* Redirects subsequent work to another stream of the same device. */
int synk_context_set_stream(synk_context *ctx, void *stream);
/* Waits for the context's stream; returns SYNK_ETIMEOUT if a persistent
 * kernel gave up at a grid barrier, SYNK_ECUDA on an asynchronous CUDA error. */
int synk_context_sync(synk_context *ctx);
/* Time limit of every wait inside the library's persistent kernels (the SIRT
 * grid barrier, the tensor-core engine's mbarrier waits): default 2 s, range
 * [1 us, 60 s].  A wait that runs out records SYNK_ETIMEOUT, its kernel
 * returns, and the next synk_context_sync() reports it and clears it.
 * missing_blocks > 0 is fault injection for testing that path: the grid
 * barrier of the next persistent SIRT launches waits for that many blocks
 * more than were launched, so every barrier runs out after timeout_ns.  Pass
 * 0 in production.  No reference counterpart: the reference surfaces failures
 * only as the runtime's error codes (futhark's context error string). */
int synk_context_set_barrier_limit(synk_context *ctx, uint64_t timeout_ns, int32_t missing_blocks);
/* Message of the last failure on this context ("" when none).  The pointer
 * stays valid until the next call on the context. */
const char *synk_context_get_error(synk_context *ctx);
/* Library version string. */
const char *synk_version(void);

/* ---- entry points of the reference programs ---- */

/* futhark/forwardprojection.fut:71-84 `main (angles, rhozero, deltarho,
 * numrhos, image)`: out[a*numrhos] = angle-major sinogram of the
 * size x size image, size = sqrt(n). */
int synk_forwardprojection(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                           float deltarho, int32_t numrhos, const float *image, int64_t n);

/* futhark/forwardprojection_sparse.fut:26-40: the same program, benchmarked by
 * the reference on sparse-view (1..95 angle) datasets. */
int synk_forwardprojection_sparse(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                                  float deltarho, int32_t numrhos, const float *image, int64_t n);

/* futhark/backprojection.fut:82-93 `main (angles, rhozero, deltarho, size,
 * projections)`: out[size*size] = backprojection of projections[p],
 * numrhos = p / a. */
int synk_backprojection(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                        float deltarho, int32_t size, const float *projections, int64_t p);

/* futhark/backprojection_sparse.fut:26-37: same program, sparse-view datasets. */
int synk_backprojection_sparse(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                               float deltarho, int32_t size, const float *projections, int64_t p);

/* futhark/SIRT.fut:43-49 `main (angles, rhozero, deltarho, image,
 * projections, iterations)`: out[n] = `iterations` SIRT updates
 * x <- x + C*BP(R*(b - FP(x))) starting from image[n] (SIRT.fut:9-41). */
int synk_SIRT(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero, float deltarho,
              const float *image, int64_t n, const float *projections, int64_t p, int32_t iterations);

/* futhark/SIRT3D.fut:18-29 `main (angles, rhos, projections, iterations,
 * size)`: `size` independent slices (zero start), slice i reconstructed from
 * projections[i*r*a : (i+1)*r*a]; out[size*size*size].  rhozero = rhos[0],
 * deltarho = rhos[1] - rhos[0] (the convention of
 * archive/projection_lib.fut:114-115; the reference's own call passes rhos
 * where SIRT expects those two scalars). */
int synk_SIRT3D(synk_context *ctx, float *out, const float *angles, int64_t a, const float *rhos, int64_t r,
                const float *projections, int64_t p, int32_t iterations, int32_t size);

/* ---- extended SIRT (no reference counterpart: stopping rule, history) ---- */

typedef struct synk_sirt_options {
    /* Stop once ||FP(x_k) - b|| / ||b|| <= tol (0 = run all iterations).  The
     * residual of x_k is measured in the forward pass of iteration k. */
    double tol;
    /* Optional DEVICE array [iterations+1] (per slice: [nslices][iterations+1])
     * receiving ||FP(x_k) - b|| / ||b|| for k = 0..iterations (entries after a
     * stop stay as they were).  NULL = not recorded. */
    double *residuals;
    /* Optional DEVICE array [nslices] receiving the number of updates applied. */
    int32_t *iterations_done;
    /* Rows (FP) / angles (BP) split per work item: 0 = automatic. */
    int32_t fp_split;
    int32_t bp_split;
    /* Engine and grid: > 0 = the persistent kernel with that many blocks;
     * 0 = automatic (one launch per phase and iteration for a single problem,
     * and for batches whose iteration is small: at most 6e7 ray-row steps plus
     * pixel-angle pairs; otherwise the persistent kernel with every block that
     * fits); -1 = one launch per phase and iteration.  With tol > 0 the
     * launch loop ends early: every 16 iterations the call reads the number of
     * slices still updating, which waits for the stream (not while the stream
     * is being captured into a graph; the loop then runs to the end, each
     * launch doing nothing once every slice has stopped). */
    int32_t grid_blocks;
} synk_sirt_options;

/* SIRT of `nslices` independent slices sharing one geometry in ONE persistent
 * launch: image/out/projections hold nslices consecutive slices ([nslices*n]
 * and [nslices*p]); image may be NULL for a zero start. */
int synk_sirt_slices(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                     float deltarho, int32_t numrhos, int32_t size, int32_t nslices, const float *image,
                     const float *projections, int32_t iterations, const synk_sirt_options *opts);

/* Independent SIRT problems of any sizes in ONE persistent launch (no
 * reference counterpart; SIRT3D is the special case of one problem with many
 * slices).  Each problem is a stack of `nslices` slices sharing one geometry.
 * All arrays are device pointers: image [nslices*size*size] (NULL = zero
 * start), projections [nslices*a*numrhos], out [nslices*size*size],
 * residuals (optional) [nslices][iterations+1], iterations_done (optional)
 * [nslices]. */
typedef struct synk_sirt_problem {
    const float *angles;
    int64_t a;
    float rhozero;
    float deltarho;
    int32_t numrhos;
    int32_t size;
    int32_t nslices;
    int32_t iterations;
    const float *image;
    const float *projections;
    float *out;
    double *residuals;
    int32_t *iterations_done;
    int32_t fp_split;   /* 0 = automatic */
    int32_t bp_split;   /* 0 = automatic */
} synk_sirt_problem;

/* Blocks of the persistent SIRT kernel that fit on the current device at once
 * (the largest useful grid_blocks); 0 if it cannot be resident. */
int synk_sirt_resident_blocks(void);

/* tol and grid_blocks as in synk_sirt_options. */
int synk_sirt_batch(synk_context *ctx, int32_t nprob, const synk_sirt_problem *probs, double tol,
                    int32_t grid_blocks);

/* A batched SIRT solve captured once in a CUDA graph (with its own scratch)
 * and replayed by synk_sirt_plan_launch on the context's stream.  The arrays
 * of `probs` are bound at creation: change their contents between launches,
 * not the pointers.  grid_blocks 0 selects the persistent kernel here (a
 * captured phase-split loop cannot end early); -1 captures one launch per
 * phase and iteration. */
typedef struct synk_sirt_plan synk_sirt_plan;
int synk_sirt_plan_new(synk_context *ctx, synk_sirt_plan **out, int32_t nprob, const synk_sirt_problem *probs,
                       double tol, int32_t grid_blocks);
int synk_sirt_plan_launch(synk_context *ctx, synk_sirt_plan *plan);
void synk_sirt_plan_free(synk_sirt_plan *plan);

/* ---- CSR system matrix (no reference counterpart) ----
 * The forward projector's rule (futhark/forwardprojection.fut:31-56) stored
 * as a sparse matrix A (rows: rays k*numrhos + r, angle-major; columns:
 * row-major pixels) together with its exact transpose A^T, both built on the
 * GPU.  Row pointers are int64, column indices int32, values float32. */
typedef struct synk_csr synk_csr;

int synk_csr_new(synk_context *ctx, synk_csr **out, const float *angles, int64_t a, float rhozero, float deltarho,
                 int32_t numrhos, int32_t size);
void synk_csr_free(synk_csr *m);
/* rows = a*numrhos, cols = size*size, nnz = non-zeros of A (= of A^T). */
int synk_csr_shape(const synk_csr *m, int64_t *rows, int64_t *cols, int64_t *nnz);
/* Device arrays of A (transpose = 0) or A^T (transpose = 1). */
int synk_csr_arrays(const synk_csr *m, int transpose, const int64_t **rowptr, const int32_t **colidx,
                    const float **vals);
/* y[rows] = A x[cols] */
int synk_csr_spmv(synk_context *ctx, const synk_csr *m, const float *x, float *y);
/* x[cols] = A^T y[rows] */
int synk_csr_spmv_t(synk_context *ctx, const synk_csr *m, const float *y, float *x);
/* y[rows] = M x for a caller-owned CSR matrix (int32 row pointers). */
int synk_spmv_csr32(synk_context *ctx, int64_t rows, const int32_t *rowptr, const int32_t *colidx,
                    const float *vals, const float *x, float *y);

/* ---- the reference's validation programs (futhark/tools/*.fut) ----
 * One pass over two float32 device arrays of n elements:
 *   count  = #{ i > 0 : |sane[i] - test[i]| > tol }   (tools/diff.fut:4-6, tol 0.05)
 *   sse    = sum (sane[i] - test[i])^2, FP64           (tools/mse.fut:2-3)
 *   all_ok = every |sane[i] - test[i]| < tol           (tools/sanityCheck.fut:3-4)
 * `out` points to device memory.  synk_diff / synk_mse / synk_sanityCheck
 * write the reference programs' own results to a device scalar: an int32
 * count, the float32 mean sse/n and a one-byte boolean; the tolerance is the
 * programs' std_dev = 0.05. */
typedef struct {
    uint64_t count;
    double sse;
    int32_t all_ok;
    int32_t pad_;
} synk_compare_result;
int synk_compare(synk_context *ctx, synk_compare_result *out, const float *sane, const float *test, int64_t n,
                 float tol);
int synk_diff(synk_context *ctx, int32_t *out, const float *sane, const float *test, int64_t n);
int synk_mse(synk_context *ctx, float *out, const float *sane, const float *test, int64_t n);
int synk_sanityCheck(synk_context *ctx, uint8_t *out, const float *sane, const float *test, int64_t n);

/* ---- backprojection that allocates nothing (no counterpart in the reference) ----
 * For callers that cannot let the library allocate device memory: programs
 * that reserve all free device memory for their own allocator at start-up,
 * and acquisition loops that must not enter the CUDA allocator while frames
 * stream (an allocation can take the driver's allocator lock or synchronise
 * the device).  Same arguments and result as synk_backprojection, at most
 * SYNK_NOALLOC_MAX_ANGLES angles (larger counts return SYNK_EINVAL).  Its
 * scratch is one file-scope device array (about 448 KiB) that every GPU
 * loading the library holds until exit.  The first call on a device looks up
 * that array's device address (cudaGetSymbolAddress) and keeps it for the
 * life of the process; make that first call before any stream capture.  A
 * device reset (cudaDeviceReset) invalidates the kept address: this entry
 * point does not support a reset of a device it has run on.  All calls share
 * the array: calls that overlap on the GPU race and must be serialised by the
 * caller. */
#define SYNK_NOALLOC_MAX_ANGLES 8192
int synk_backprojection_noalloc(synk_context *ctx, float *out, const float *angles, int64_t a, float rhozero,
                                float deltarho, int32_t size, const float *projections, int64_t p);

/* ---- BF16 tensor-core building blocks of the U-Net warm starter (no reference
 * counterpart).  BF16 arrays are passed as uint16_t bit patterns, NHWC. ---- */

/* C[M x N] (FP32) = A[M x K] * B[N x K]^T, A and B BF16 row-major (K
 * contiguous).  M % 128 == 0, 16 <= N <= 256, N % 16 == 0, K % 64 == 0. */
int synk_gemm_bf16(synk_context *ctx, const uint16_t *A, const uint16_t *B, float *C, int32_t M, int32_t N,
                   int32_t K);

/* 3x3 convolution, padding 1: y[b,h,w,yoff+o] = epi(sum_{tap,i} x[b,h+ky-1,w+kx-1,xoff+i]
 * * w[o][(ky*3+kx)*Cin + i]) with x [B][H][W][ldx], y [B][H][W][ldy], w [Cout][9*Cin].
 * epi: 1 = relu(. + bias), 4 = . + bias, 2 = . * (mask[b,h,w,moff+o] > 0).
 * Cin % 32 == 0, Cout % 16 == 0, Cout <= 256, H*W a multiple of 128 tiles. */
int synk_conv3x3_bf16(synk_context *ctx, const uint16_t *x, int32_t ldx, int32_t xoff, int32_t Cin, int32_t B,
                      int32_t H, int32_t W, const uint16_t *w, const float *bias, uint16_t *y, int32_t ldy,
                      int32_t yoff, int32_t Cout, int32_t epi, const uint16_t *mask, int32_t ldm, int32_t moff);

/* dw[o][tap*Cin + i] += sum_p dy[p][o] * x[p + tap][i] from blocked copies
 * with pixel chunks of c = 64 (W >= 64) or 32 pixels of one image row:
 * dyT [B][H][W/c][Cout][c] and the three W-shifted copies
 * xT3 [3][B][H][W/c][Cin][c] (copy k holds x[w + k - 1], zero outside the
 * row); dw FP32 [Cout][9*Cin]. */
int synk_conv3x3_wgrad_bf16(synk_context *ctx, const uint16_t *dyT, const uint16_t *xT3, float *dw, int32_t Cin,
                            int32_t Cout, int32_t B, int32_t H, int32_t W, int32_t ksplit);

/* ---- U-Net warm starter (no reference counterpart) ----
 * 4 levels, 32 base channels, 3x3 convolutions + ReLU, BF16 activations, FP32
 * accumulation and FP32 master weights; input the normalised backprojection
 * C*A^T*R*b, output a start image for SIRT (x + a learned correction).
 * Images are FP32 [batch][size][size] device arrays; size is a multiple of 256. */
typedef struct synk_unet synk_unet;

int synk_unet_new(synk_context *ctx, synk_unet **out, int32_t max_batch, int32_t size, uint64_t seed);
void synk_unet_free(synk_unet *net);
int64_t synk_unet_num_params(const synk_unet *net);
/* direction 0: copy the FP32 parameters to dst; 1: load them from dst. */
int synk_unet_params(synk_context *ctx, synk_unet *net, float *dst, int32_t direction);
/* Adam state, for checkpoints: direction 0 copies the first and second
 * moments to the DEVICE arrays m and v ([num_params] FP32 each, the parameter
 * layout) and the number of Adam steps taken to the HOST scalar *step;
 * direction 1 loads all three, so that training resumes where it stopped. */
int synk_unet_optimizer_state(synk_context *ctx, synk_unet *net, float *m, float *v, int64_t *step,
                              int32_t direction);
/* y = net(x) for `batch` images. */
int synk_unet_forward(synk_context *ctx, synk_unet *net, const float *x, float *y, int32_t batch);
/* One training step on (x, target) with the MSE loss: forward, backward and,
 * when apply != 0, one fused Adam update with learning rate lr (beta 0.9 /
 * 0.999, eps 1e-8).  loss (optional device double) receives the batch loss. */
int synk_unet_train_step(synk_context *ctx, synk_unet *net, const float *x, const float *target, int32_t batch,
                         float lr, int32_t apply, double *loss);
/* FP32 gradients of the last train step run with apply = 0 (same layout as the parameters). */
int synk_unet_gradients(synk_context *ctx, synk_unet *net, float *dst);

#ifdef __cplusplus
}
#endif

#endif /* SYNK_H */

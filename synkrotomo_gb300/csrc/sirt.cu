// Persistent SIRT kernel (futhark/SIRT.fut:27-39 for one slice,
// futhark/SIRT3D.fut:23-28 for a stack of independent slices).
//
// One cooperative launch runs every iteration of every slice:
//   phase FP (iteration k):  e = b - FP(x_k), rr = R*e, sum e^2 (FP64)
//   grid barrier
//   phase BP (iteration k):  x_{k+1} = x_k + C*BP(rr), written to the padded
//                            image and (through shared memory) to the padded
//                            transposed image that the next FP phase reads
//   grid barrier
// Work items are assigned statically (item = block + i*grid) and are all of
// one size within a phase.  The grid barrier spins with a time limit; a block
// that gives up records SYNK_ETIMEOUT in the status word and returns, after
// which every other block gives up at its next barrier too.
#include <math.h>

#include "synk_internal.cuh"
#include "sirt_internal.cuh"
#include "fp_tile.cuh"
#include "bp_tile.cuh"

namespace synk {

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned *p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acqrel_u32(unsigned *p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier with a time limit.  Returns false (in every thread of the
// block) once the barrier or any other block has failed.
__device__ bool grid_barrier(unsigned *bar, unsigned nblocks, int *status, unsigned long long timeout_ns,
                             int *s_flag) {
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned gen = ld_acquire_u32(&bar[1]);
        const unsigned arrived = atom_add_acqrel_u32(&bar[0], 1u);
        if (arrived == nblocks - 1u) {
            atomicExch(&bar[0], 0u);
            st_release_u32(&bar[1], gen + 1u);
        } else {
            const unsigned long long t0 = global_ns();
            for (unsigned spin = 0;; ++spin) {
                if (ld_acquire_u32(&bar[1]) != gen) break;
                if ((spin & 15u) == 15u) {
                    if (global_ns() - t0 > timeout_ns || spin > (1u << 30)) {
                        atomicExch(status, SYNK_ETIMEOUT);
                        ok = 0;
                        break;
                    }
                }
                __nanosleep(20);
            }
        }
        if (ok && *(volatile int *)status != 0) ok = 0;
        *s_flag = ok;
    }
    __syncthreads();
    return *s_flag != 0;
}

__device__ __forceinline__ bool slice_active(const SirtParams &p, int s, int it) {
    if (p.tol2 <= 0.0) return true;
    if (*(volatile const int *)(p.stop_iter + s) < it) return false;
    const double r2 = *(volatile const double *)(p.res2 + (size_t)s * (p.iterations + 1) + it);
    return !(r2 <= p.tol2 * p.b2[s]);
}

__device__ __forceinline__ double warp_sum_d(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

struct SirtShared {
    BpStage st;
    float red[8][33];
    float red4[8][4][32];
    float tile[32][33];
    double e2;
    int flag;
    int any;
};

__device__ __forceinline__ void flush_e2(const SirtParams &p, int it, int slice, SirtShared &sh) {
    if (threadIdx.x == 0 && slice >= 0) {
        atomicAdd(p.res2 + (size_t)slice * (p.iterations + 1) + it, sh.e2);
        sh.e2 = 0.0;
    }
}

// residual of one ray: e = b - fp; rr = R*e (SIRT.fut:33-36); returns e^2
__device__ __forceinline__ double residual(const SirtParams &p, int s, int k, int r, float fpv) {
    const size_t pr = (size_t)p.P.a * p.P.D;
    const size_t ray = (size_t)k * p.P.D + r;
    const float e = __fsub_rn(p.b[(size_t)s * pr + ray], fpv);
    p.rr[(size_t)s * pr + ray] = __fmul_rn(p.R[ray], e);
    return (double)e * (double)e;
}

// ---- phase FP of iteration `it` ------------------------------------------------
__device__ void fp_phase(const SirtParams &p, int it, SirtShared &sh) {
    const ProbGeom &P = p.P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int S = p.fp_split, G = 8 / S;                 // G detectors per item, S row parts
    const int ngroups = __ldg(p.L.counts) + __ldg(p.L.counts + 1);
    const int nsteep = __ldg(p.L.counts);
    const int nexact = __ldg(p.L.counts + 2);
    const int dblocks = (P.D + G - 1) / G;
    const int fast_items = ngroups * dblocks;
    const int etiles = (P.D + 255) / 256;
    const int ips = fast_items + nexact * etiles;      // items per slice
    const int total = ips * p.nslices;
    const size_t np = (size_t)P.N * (P.N + 2);
    const int part = warp % S;
    const int jb = (int)((long long)part * P.N / S), je = (int)((long long)(part + 1) * P.N / S);
    int cur_slice = -1;
    if (threadIdx.x == 0) sh.e2 = 0.0;
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        const int s = item / ips;
        const int rem = item - s * ips;
        __syncthreads();                                  // red / e2 reuse
        if (s != cur_slice) {
            flush_e2(p, it, cur_slice, sh);
            cur_slice = s;
        }
        if (p.tol2 > 0.0 && *(volatile const int *)(p.stop_iter + s) < it) continue;   // slice finished earlier
        double e2 = 0.0;
        if (rem < fast_items) {
            const int grp = rem / dblocks;
            const int db = rem - grp * dblocks;
            const int r = db * G + warp / S;
            const int k = r < P.D ? __ldg(p.L.order + grp * 32 + lane) : -1;
            const float *img = (grp < nsteep ? p.xpad : p.xTpad) + (size_t)s * np;
            const float v = fp_lane_ray(P, k, r, img, jb, je);
            sh.red[warp][lane] = v;
            __syncthreads();
            if (part == 0 && k >= 0) {
                float fpv = sh.red[warp][lane];
                for (int q = 1; q < S; ++q) fpv += sh.red[warp + q][lane];
                e2 = residual(p, s, k, r, fpv);
            }
        } else {
            const int x = rem - fast_items;
            const int e = x / etiles;
            const int r = (x - e * etiles) * 256 + threadIdx.x;
            if (r < P.D) {
                const int k = __ldg(p.L.exact + e);
                const float v = fp_exact_ray(P, k, r, p.xpad + (size_t)s * np, p.xTpad + (size_t)s * np);
                e2 = residual(p, s, k, r, v);
            }
        }
        e2 = warp_sum_d(e2);
        if (lane == 0) atomicAdd(&sh.e2, e2);
    }
    __syncthreads();
    flush_e2(p, it, cur_slice, sh);
}

// ---- phase BP of iteration `it` ------------------------------------------------
__device__ void bp_phase(const SirtParams &p, int it, SirtShared &sh) {
    const ProbGeom &P = p.P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int SB = p.bp_split, RB = 8 / SB;     // angle parts, warp rows
    const int TR = 4 * RB;                      // tile rows
    const int tx_n = (P.N + 31) / 32, ty_n = (P.N + TR - 1) / TR;
    const int ips = tx_n * ty_n;
    const int total = ips * p.nslices;
    const size_t pr = (size_t)P.a * P.D, np = (size_t)P.N * (P.N + 2);
    const int wrow = warp / SB, part = warp % SB;
    const int nexact = __ldg(p.L.counts + 2);
    const bool unit = P.deltarho == 1.0f;
    for (int item = blockIdx.x; item < total; item += gridDim.x) {
        const int s = item / ips;
        const int rem = item - s * ips;
        const int ty = rem / tx_n;
        const int tx = rem - ty * tx_n;
        if (!slice_active(p, s, it)) continue;      // uniform over the block
        const int col = tx * 32 + lane;
        const int row0 = ty * TR + wrow;
        const float xc = (float)(col - P.half) + 0.5f;
        const float yc0 = (float)(row0 - P.half) + 0.5f;
        const float *rr = p.rr + (size_t)s * pr;
        float sum[4] = {0.0f, 0.0f, 0.0f, 0.0f}, comp[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        for (int kc = 0; kc < P.a; kc += kBpChunk) {
            __syncthreads();
            bp_stage(P, kc, sh.st);
            __syncthreads();
            float prt[4] = {0.0f, 0.0f, 0.0f, 0.0f};
            if (unit) bp_chunk<4, true>(P, sh.st, kc, P.a, part, SB, rr, xc, yc0, (float)RB, prt);
            else bp_chunk<4, false>(P, sh.st, kc, P.a, part, SB, rr, xc, yc0, (float)RB, prt);
#pragma unroll
            for (int m = 0; m < 4; ++m) comp_add(sum[m], comp[m], prt[m]);
        }
        float ex[4] = {0.0f, 0.0f, 0.0f, 0.0f};
        bp_exact_angles<4>(P, p.L.exact, nexact, part, SB, rr, row0, RB, col, ex);
#pragma unroll
        for (int m = 0; m < 4; ++m) sh.red4[warp][m][lane] = (sum[m] + comp[m]) + ex[m];
        __syncthreads();
        float *xpad = p.xpad + (size_t)s * np;
        if (part == 0) {
#pragma unroll
            for (int m = 0; m < 4; ++m) {
                float bpv = sh.red4[warp][m][lane];
                for (int q = 1; q < SB; ++q) bpv += sh.red4[warp + q][m][lane];
                const int row = row0 + RB * m;
                float xi = 0.0f;
                if (row < P.N && col < P.N) {
                    const size_t pix = (size_t)row * P.N + col;
                    float *xp = xpad + (size_t)row * (P.N + 2) + col + 1;
                    xi = __fadd_rn(*xp, __fmul_rn(p.C[pix], bpv));             // SIRT.fut:38-39
                    *xp = xi;
                }
                sh.tile[lane][wrow + RB * m] = xi;
            }
        }
        __syncthreads();
        // transposed write: xTpad[col][row + 1] for the tile's 32 columns x TR rows
        float *xTpad = p.xTpad + (size_t)s * np;
        for (int i = threadIdx.x; i < 32 * TR; i += blockDim.x) {
            const int cl = i / TR, rl = i - cl * TR;
            const int c = tx * 32 + cl, r = ty * TR + rl;
            if (c < P.N && r < P.N) xTpad[(size_t)c * (P.N + 2) + r + 1] = sh.tile[cl][rl];
        }
    }
}

__global__ void __launch_bounds__(256, 2) sirt_persistent_kernel(SirtParams p) {
    __shared__ SirtShared sh;
    const unsigned nb = gridDim.x;
    for (int it = 0; it <= p.iterations; ++it) {
        const bool final_fp = it == p.iterations;
        if (final_fp && !p.record_final) break;
        fp_phase(p, it, sh);
        if (!grid_barrier(p.bar, nb, p.status, p.timeout_ns, &sh.flag)) return;
        if (final_fp) break;
        // stopping rule (identical decision in every block)
        if (p.tol2 > 0.0) {
            if (threadIdx.x == 0) sh.any = 0;
            __syncthreads();
            for (int s = threadIdx.x; s < p.nslices; s += blockDim.x) {
                if (slice_active(p, s, it)) sh.any = 1;
                else if (blockIdx.x == 0 && p.stop_iter[s] >= p.iterations) p.stop_iter[s] = it;
            }
            __syncthreads();
            if (!sh.any) break;
        }
        bp_phase(p, it, sh);
        if (!grid_barrier(p.bar, nb, p.status, p.timeout_ns, &sh.flag)) return;
    }
}

// ||b_s||^2 per slice in FP64.
__global__ void sumsq_kernel(const float *__restrict__ b, size_t len, double *__restrict__ out) {
    const int s = blockIdx.y;
    const float *bs = b + (size_t)s * len;
    double acc = 0.0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < len; i += (size_t)gridDim.x * blockDim.x)
        acc += (double)bs[i] * (double)bs[i];
    acc = warp_sum_d(acc);
    __shared__ double shd[32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) shd[w] = acc;
    __syncthreads();
    if (w == 0) {
        acc = l < (int)(blockDim.x >> 5) ? shd[l] : 0.0;
        acc = warp_sum_d(acc);
        if (l == 0) atomicAdd(out + s, acc);
    }
}

// residuals[s][k] = sqrt(res2[s][k] / b2[s]); iterations_done[s].
__global__ void sirt_finalize_kernel(SirtParams p, double *residuals, int *iters_done) {
    const int s = blockIdx.x;
    const int K = p.iterations + 1;
    const int stop = p.stop_iter[s] < p.iterations ? p.stop_iter[s] : p.iterations;
    if (threadIdx.x == 0 && iters_done) iters_done[s] = stop;
    if (!residuals) return;
    const int last = p.record_final ? p.iterations : p.iterations - 1;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        if (k > stop || k > last) continue;
        const double b2 = p.b2[s];
        residuals[(size_t)s * K + k] = b2 > 0.0 ? sqrt(p.res2[(size_t)s * K + k] / b2) : 0.0;
    }
}

cudaError_t launch_sumsq(const float *b, size_t len, int nslices, double *out, cudaStream_t stream) {
    dim3 grid(64, nslices);
    sumsq_kernel<<<grid, 256, 0, stream>>>(b, len, out);
    return cudaGetLastError();
}

int sirt_persistent_grid(int *blocks_per_sm) {
    int dev = 0, sms = 0, bps = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, sirt_persistent_kernel, 256, 0);
    if (blocks_per_sm) *blocks_per_sm = bps;
    return sms * bps;
}

cudaError_t launch_sirt_persistent(const SirtParams &p, int grid, cudaStream_t stream) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, sirt_persistent_kernel, p);
}

cudaError_t launch_sirt_finalize(const SirtParams &p, double *residuals, int *iters_done, cudaStream_t stream) {
    sirt_finalize_kernel<<<p.nslices, 128, 0, stream>>>(p, residuals, iters_done);
    return cudaGetLastError();
}

}  // namespace synk

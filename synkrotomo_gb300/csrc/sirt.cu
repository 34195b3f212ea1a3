// Persistent SIRT kernel (futhark/SIRT.fut:27-39 for one slice,
// futhark/SIRT3D.fut:23-28 for a stack of independent slices).
//
// One cooperative launch runs every iteration of every slice:
//   phase FP (iteration k):  e = b - FP(x_k), rr = R*e, sum e^2 (FP64)
//   grid barrier
//   phase BP (iteration k):  x_{k+1} = x_k + C*BP(rr), also written transposed
//   grid barrier
// Work items are handed out by an atomic counter (three counters rotate over
// the phases), so slices of any number share the whole GPU.  The grid
// barrier spins with a time limit; a block that gives up records
// SYNK_ETIMEOUT in the status word and returns, after which every other block
// gives up at its next barrier too.
#include <math.h>

#include "synk_internal.cuh"
#include "sirt_internal.cuh"

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
                if ((spin & 31u) == 31u) {
                    if (global_ns() - t0 > timeout_ns || spin > (1u << 30)) {
                        atomicExch(status, SYNK_ETIMEOUT);
                        ok = 0;
                        break;
                    }
                }
                __nanosleep(32);
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

__device__ __forceinline__ int next_item(unsigned *counter, int *s_item) {
    __syncthreads();
    if (threadIdx.x == 0) *s_item = (int)atomicAdd(counter, 1u);
    __syncthreads();
    return *s_item;
}

// ---- phase FP of iteration `it` ------------------------------------------------
__device__ void fp_phase(const SirtParams &p, int it, unsigned *counter, float (*red)[33], int *s_item,
                         double *s_e2) {
    const ProbGeom &P = p.P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int S = p.fp_split, G = 8 / S;
    const int tiles = (P.D + 31) / 32;
    const int groups = (P.a + G - 1) / G;
    const int ips = tiles * groups;
    const int total = ips * p.nslices;
    const size_t n = (size_t)P.N * P.N, pr = (size_t)P.a * P.D;
    const int part = warp % S;
    const int jb = (int)((long long)part * P.N / S), je = (int)((long long)(part + 1) * P.N / S);
    int cur_slice = -1;
    if (threadIdx.x == 0) *s_e2 = 0.0;
    for (;;) {
        const int item = next_item(counter, s_item);
        if (item >= total) break;
        const int s = item / ips;
        const int rem = item - s * ips;
        const int kg = rem / tiles;
        const int t = rem - kg * tiles;
        if (s != cur_slice) {
            if (threadIdx.x == 0 && cur_slice >= 0) {
                atomicAdd(p.res2 + (size_t)cur_slice * (p.iterations + 1) + it, *s_e2);
                *s_e2 = 0.0;
            }
            cur_slice = s;
        }
        // a slice whose stopping rule fired at an earlier iteration is done
        if (p.tol2 > 0.0 && *(volatile const int *)(p.stop_iter + s) < it) continue;
        const int k = kg * G + warp / S;
        const int r = t * 32 + lane;
        float v = 0.0f;
        if (k < P.a && r < P.D) {
            const AngleGeom g = load_geom(P.geom, k);
            const float *frame = (g.flat ? p.xT : p.x) + (size_t)s * n;
            v = fp_ray<false>(P, g, frame, r, jb, je);
        }
        red[warp][lane] = v;
        __syncthreads();
        double e2 = 0.0;
        if (part == 0 && k < P.a && r < P.D) {
            float fpv = red[warp][lane];
            for (int q = 1; q < S; ++q) fpv += red[warp + q][lane];
            const size_t ray = (size_t)k * P.D + r;
            const float e = __fsub_rn(p.b[(size_t)s * pr + ray], fpv);            // SIRT.fut:33-34
            p.rr[(size_t)s * pr + ray] = __fmul_rn(p.R[ray], e);                  // SIRT.fut:35-36
            e2 = (double)e * (double)e;
        }
        e2 = warp_sum_d(e2);
        if (lane == 0 && part == 0) atomicAdd(s_e2, e2);
    }
    __syncthreads();
    if (threadIdx.x == 0 && cur_slice >= 0) atomicAdd(p.res2 + (size_t)cur_slice * (p.iterations + 1) + it, *s_e2);
}

// ---- phase BP of iteration `it` ------------------------------------------------
__device__ void bp_phase(const SirtParams &p, int it, unsigned *counter, float (*red)[33], int *s_item) {
    const ProbGeom &P = p.P;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int SB = p.bp_split, RB = 8 / SB;
    const int tx_n = (P.N + 31) / 32, ty_n = (P.N + RB - 1) / RB;
    const int ips = tx_n * ty_n;
    const int total = ips * p.nslices;
    const size_t n = (size_t)P.N * P.N, pr = (size_t)P.a * P.D;
    const int part = warp % SB;
    const int ka = (int)((long long)part * P.a / SB), kb = (int)((long long)(part + 1) * P.a / SB);
    for (;;) {
        const int item = next_item(counter, s_item);
        if (item >= total) break;
        const int s = item / ips;
        const int rem = item - s * ips;
        const int ty = rem / tx_n;
        const int tx = rem - ty * tx_n;
        if (!slice_active(p, s, it)) continue;
        const int row = ty * RB + warp / SB;
        const int col = tx * 32 + lane;
        float v = 0.0f;
        if (row < P.N && col < P.N) {
            const float *rr = p.rr + (size_t)s * pr;
            float sum = 0.0f, comp = 0.0f;
            for (int k0 = ka; k0 < kb; k0 += 32) {
                const int k1 = min(k0 + 32, kb);
                float partial = 0.0f;
                for (int k = k0; k < k1; ++k) {
                    const AngleGeom g = load_geom(P.geom, k);
                    partial += bp_angle<false>(P, g, rr + (size_t)k * P.D, row, col);
                }
                comp_add(sum, comp, partial);
            }
            v = sum + comp;
        }
        red[warp][lane] = v;
        __syncthreads();
        if (part == 0 && row < P.N && col < P.N) {
            float bpv = red[warp][lane];
            for (int q = 1; q < SB; ++q) bpv += red[warp + q][lane];
            const size_t pix = (size_t)row * P.N + col;
            float *x = p.x + (size_t)s * n;
            const float xi = __fadd_rn(x[pix], __fmul_rn(p.C[pix], bpv));        // SIRT.fut:38-39
            x[pix] = xi;
            p.xT[(size_t)s * n + (size_t)col * P.N + row] = xi;
        }
    }
}

__global__ void __launch_bounds__(256, 2) sirt_persistent_kernel(SirtParams p) {
    __shared__ float red[8][33];
    __shared__ int s_item;
    __shared__ int s_flag;
    __shared__ double s_e2;
    const unsigned nb = gridDim.x;
    for (int it = 0; it <= p.iterations; ++it) {
        const bool final_fp = it == p.iterations;
        if (final_fp && !p.record_final) break;
        // phase 2*it: FP.  Reset the counter of the phase after next.
        const int ph = 2 * it;
        if (blockIdx.x == 0 && threadIdx.x == 0) p.work[(ph + 1) % 3] = 0u;
        fp_phase(p, it, p.work + ph % 3, red, &s_item, &s_e2);
        if (!grid_barrier(p.bar, nb, p.status, p.timeout_ns, &s_flag)) return;
        if (final_fp) break;
        // stopping rule (identical decision in every block)
        if (p.tol2 > 0.0) {
            __shared__ int s_any;
            if (threadIdx.x == 0) s_any = 0;
            __syncthreads();
            for (int s = threadIdx.x; s < p.nslices; s += blockDim.x) {
                if (slice_active(p, s, it)) s_any = 1;
                else if (blockIdx.x == 0 && p.stop_iter[s] >= p.iterations) p.stop_iter[s] = it;
            }
            __syncthreads();
            if (!s_any) break;
        }
        const int ph2 = ph + 1;
        if (blockIdx.x == 0 && threadIdx.x == 0) p.work[(ph2 + 1) % 3] = 0u;
        bp_phase(p, it, p.work + ph2 % 3, red, &s_item);
        if (!grid_barrier(p.bar, nb, p.status, p.timeout_ns, &s_flag)) return;
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
    __shared__ double sh[32];
    const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
    if (l == 0) sh[w] = acc;
    __syncthreads();
    if (w == 0) {
        acc = l < (int)(blockDim.x >> 5) ? sh[l] : 0.0;
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

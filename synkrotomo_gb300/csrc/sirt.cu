// SIRT engines (futhark/SIRT.fut:27-39 per slice; futhark/SIRT3D.fut:23-28 for
// slice stacks; any number of independent problems of uneven size).
//
// Persistent engine: one cooperative launch runs every iteration of every problem:
//   phase FP (iteration k):  e = b - FP(x_k), rr = R*e, sum e^2 (FP64)
//   grid barrier
//   phase BP (iteration k):  x_{k+1} = x_k + C*BP(rr), written to the padded
//                            image and (through shared memory) to the padded
//                            transposed image that the next FP phase reads
//   grid barrier
// Problems carry their own geometry, work split and iteration count; a
// problem past its count (or stopped by the residual rule) drops out of both
// phases.  Items of one problem: FP = (slice, angle group, detector block) and
// (slice, near-axis angle, 8 detectors); BP = (slice, 32-column tile).  A
// single problem uses a static assignment (item = block + i*grid); a batch is
// handed out by an atomic counter, largest problems first.  The grid barrier
// spins with a time limit; a block that gives up records SYNK_ETIMEOUT in the
// status word and returns, after which every other block gives up at its next
// barrier too.
//
// The phase-split engine runs the same phases as ordinary launches, one per
// phase and iteration (the kernel boundary replaces the barrier); for a single
// problem its forward phase runs on the projector's own grid
// (sirt_fp_stack_kernel).  The host picks the engine (capi.cu, sirt_batch).
#include <limits.h>
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
    double e2w[8];        // per-warp e^2 partials of a flush
    long long item;
    int flag;
    int any;
};

__device__ __forceinline__ int stop_of(const SirtProblem &q, int s) {
    return *(volatile const int *)(q.stop_iter + s);
}
__device__ __forceinline__ double res2_of(const SirtProblem &q, int s, int it) {
    return *(volatile const double *)(q.res2 + (size_t)s * (q.iterations + 1) + it);
}

// FP of iteration it is needed when the slice has not stopped before it and
// it is at most the problem's last update (the final FP only measures).
__device__ __forceinline__ bool fp_needed(const SirtParams &p, const SirtProblem &q, int s, int it) {
    if (it > q.iterations || (it == q.iterations && !p.record_final)) return false;
    return !(p.tol2 > 0.0 && stop_of(q, s) < it);
}
// BP (the update) of iteration it: the slice is below its count and neither
// stopped before nor converged at x_it.
__device__ __forceinline__ bool bp_needed(double tol2, const SirtProblem &q, int s, int it) {
    if (it >= q.iterations) return false;
    if (tol2 <= 0.0) return true;
    if (stop_of(q, s) < it) return false;
    return !(res2_of(q, s, it) <= tol2 * q.b2[s]);
}
__device__ __forceinline__ bool bp_needed(const SirtParams &p, const SirtProblem &q, int s, int it) {
    return bp_needed(p.tol2, q, s, it);
}

// Next item of a phase: static (block + i*grid) or from the phase's counter.
__device__ __forceinline__ long long next_item(const SirtParams &p, unsigned *counter, long long prev,
                                               SirtShared &sh) {
    if (!p.dynamic) return prev < 0 ? (long long)blockIdx.x : prev + gridDim.x;
    __syncthreads();
    if (threadIdx.x == 0) sh.item = (long long)atomicAdd(counter, 1u);
    __syncthreads();
    return sh.item;
}

// problem holding global item `item` (begin offsets ascending)
__device__ __forceinline__ int find_problem(const SirtParams &p, long long item, bool fp) {
    int lo = 0, hi = p.nprob - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        const long long b = fp ? p.probs[mid].fp_begin : p.probs[mid].bp_begin;
        if (b <= item) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// residual of one ray: e = b - fp; rr = R*e (SIRT.fut:33-36), stored times the
// row's lbase for the SCALED backprojection; returns e^2.  A negative R marks
// a ray that only clips a corner pixel: it is left to graze_ray (its rr stays
// zero, so the fast backprojection adds nothing for it).
__device__ __forceinline__ double residual(const SirtProblem &q, int s, int k, int r, float fpv) {
    const size_t pr = (size_t)q.P.a * q.P.D;
    const size_t ray = (size_t)k * q.P.D + r;
    const float Rk = q.R[ray];
    if (Rk < 0.0f) return 0.0;
    const size_t i = (size_t)s * pr + ray;
    const float e = __fsub_rn(q.b[i], fpv);
    const float v = __fmul_rn(__fmul_rn(Rk, e), row_scale(q.P.geom, k));
    q.rr[i] = v;
    if (q.rrp) {                                      // pair entries r (first half) and r-1 (second half)
        q.rrp[2 * i] = v;
        if (r > 0) q.rrp[2 * i - 1] = v;
    }
    return (double)e * (double)e;
}

// Number of listed corner-clipping rays of a problem.
__device__ __forceinline__ int graze_count(const SirtProblem &q) { return __ldg(q.goff + 4); }

// Listed corner-clipping ray gidx (flat order: corner by corner) of slice s,
// one warp; returns e^2 in lane 0.  The forward value comes from the
// reference's row expressions over the rows the ray can touch (only the
// corner pixel's row has a non-zero term, so the lanes' order of summation
// gives the f32 reference's value bit for bit), and the ray's whole
// backprojection term, chord * (R*e) as the reference forms it
// (backprojection.fut:62-64 with SIRT.fut:35-37), is stored for its corner
// pixel.
__device__ __forceinline__ double graze_ray(const SirtProblem &q, int s, int gidx) {
    int c = 0;
    while (c < 3 && gidx >= __ldg(q.goff + c + 1)) ++c;
    const int slot = c * q.graze_capc + (gidx - __ldg(q.goff + c));
    const int2 ent = __ldg(q.graze + slot);
    const int k = ent.x, r = ent.y;
    const AngleGeom g = load_geom(q.P.geom, k);
    const float rho = __fadd_rn(q.P.rhozero, __fmul_rn((float)r, q.P.deltarho));
    int j0 = 0, j1 = q.P.N;
    lane_rows(q.P, g, ray_x0(g, __fdiv_rn(rho, g.cost)), j0, j1);
    const size_t np = (size_t)q.P.N * (q.P.N + 2);
    const float v = fp_exact_ray_warp(q.P, k, r, q.xpad + (size_t)s * np, q.xTpad + (size_t)s * np, j0, j1);
    double e2 = 0.0;
    if ((threadIdx.x & 31) == 0) {
        const size_t pr = (size_t)q.P.a * q.P.D;
        const size_t ray = (size_t)k * q.P.D + r;
        const float e = __fsub_rn(q.b[(size_t)s * pr + ray], v);
        q.gcontrib[(size_t)s * 4 * q.graze_capc + slot] = __fmul_rn(__ldg(q.glen + slot), __fmul_rn(-q.R[ray], e));
        e2 = (double)e * (double)e;
    }
    return e2;
}

// Backprojection terms of the listed rays that clip corner `corner` of slice
// s, summed by the calling warp (lanes over the list, combined in a fixed
// order); every lane returns the sum.
__device__ __forceinline__ float corner_terms_warp(const SirtProblem &q, int s, int corner) {
    const int lane = threadIdx.x & 31;
    const int n = __ldg(q.goff + corner + 1) - __ldg(q.goff + corner);
    const float *t = q.gcontrib + (size_t)s * 4 * q.graze_capc + (size_t)corner * q.graze_capc;
    float acc = 0.0f;
    for (int i = lane; i < n; i += 32) acc = __fadd_rn(acc, t[i]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) acc = __fadd_rn(acc, __shfl_xor_sync(0xffffffffu, acc, o));
    return acc;
}

// Adds the block's e^2 of (problem q, slice) to its residual sum: every lane
// holds a partial; the warps' sums are added in warp order.  Called by the
// whole block at block-uniform points (q and slice are uniform).
__device__ __forceinline__ void flush_e2(int it, const SirtProblem *q, int slice, double &acc, SirtShared &sh) {
    if (!q) return;
    const double w = warp_sum_d(acc);
    acc = 0.0;
    if ((threadIdx.x & 31) == 0) sh.e2w[threadIdx.x >> 5] = w;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += sh.e2w[i];
        if (t != 0.0) atomicAdd(q->res2 + (size_t)slice * (q->iterations + 1) + it, t);
    }
    // e2w is written again only after the next block-wide barrier
}

// Slice and item-in-slice of a problem-local item (32-bit division when the
// index fits).
__device__ __forceinline__ void item_slice(long long local, int ips, int &s, int &rem) {
    if (local <= 0x7fffffffLL) {
        const unsigned l = (unsigned)local, u = (unsigned)ips;
        s = (int)(l / u);
        rem = (int)(l - (unsigned)s * u);
    } else {
        s = (int)(local / ips);
        rem = (int)(local - (long long)s * ips);
    }
}

// Rows [jb, je) of part `part` of S (a power of two) equal parts of N rows.
__device__ __forceinline__ void row_part(int N, int S, int part, int &jb, int &je) {
    const int sh = __ffs(S) - 1;
    jb = (part * N) >> sh;
    je = ((part + 1) * N) >> sh;
}

// ---- phase FP of iteration `it` ------------------------------------------------
// Programmatic dependent launch: a phase kernel launched with programmatic
// stream serialization lets the next one be scheduled once all of its blocks
// have started (launch_dependents), and the next one's blocks wait in
// griddepcontrol.wait until this grid has completed and its writes are
// visible.  Every block waits before it reads anything an earlier kernel
// wrote, and before it exits, so completion stays transitive along the chain.
// Launched without the attribute both instructions return at once.
__device__ __forceinline__ void chain_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void chain_release() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// CHAINED (the chained phase kernel): the item's static setup (decode, the
// rays' geometry and row ranges, the backprojection's first angle chunk)
// runs before griddepcontrol.wait, while the previous phase finishes; every
// read of data an earlier kernel of the loop wrote (the iterate, rr, the
// residual sums, the stop iterations) comes after it.
template <bool CHAINED>
__device__ void fp_phase(const SirtParams &p, int it, unsigned *counter, SirtShared &sh) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long long total = p.totals[0];
    const SirtProblem *cur = nullptr;
    int cur_slice = -1;
    double e2acc = 0.0;                                   // this lane's e^2 of (cur, cur_slice)
    for (long long item = next_item(p, counter, -1, sh); item < total; item = next_item(p, counter, item, sh)) {
        const int qi = find_problem(p, item, true);
        const SirtProblem &q = p.probs[qi];
        const ProbGeom &P = q.P;
        int s, rem;
        item_slice(item - q.fp_begin, q.fp_ips, s, rem);
        __syncthreads();                                  // red reuse
        if (&q != cur || s != cur_slice) {
            flush_e2(it, cur, cur_slice, e2acc, sh);
            cur = &q;
            cur_slice = s;
        }
        const int S = q.fp_split, lgS = __ffs(S) - 1, G = 8 >> lgS;
        const int ngroups = __ldg(q.L.counts) + __ldg(q.L.counts + 1);
        const int nsteep = __ldg(q.L.counts);
        const int dblocks = (P.D + G - 1) >> (3 - lgS);
        const int fast_items = ngroups * dblocks;
        const size_t np = (size_t)P.N * (P.N + 2);
        double e2 = 0.0;
        if (rem < fast_items) {
            const int part = warp & (S - 1);
            int jb, je;
            row_part(P.N, S, part, jb, je);
            const int grp = (int)((unsigned)rem / (unsigned)dblocks);
            const int db = rem - grp * dblocks;
            // S = 1: 4 angles x 8 detectors per warp (as sirt_fp_stack_kernel)
            const int r = S == 1 ? db * 8 + (lane & 7) : db * G + (warp >> lgS);
            const int k = r < P.D ? __ldg(q.L.order + grp * 32 + (S == 1 ? warp * 4 + (lane >> 3) : lane)) : -1;
            const LaneRay L = lane_ray_prep(P, k, r, jb, je);
            if (CHAINED) chain_wait();
            if (!fp_needed(p, q, s, it)) continue;        // uniform over the block
            const float *img = (grp < nsteep ? q.xpad : q.xTpad) + (size_t)s * np;
            const float v = fp_lane_walk(P, L, img);
            sh.red[warp][lane] = v;
            __syncthreads();
            if (part == 0 && k >= 0) {
                float fpv = sh.red[warp][lane];
                for (int t = 1; t < S; ++t) fpv += sh.red[warp + t][lane];
                e2 = residual(q, s, k, r, fpv);
            }
        } else if (rem < fast_items + __ldg(q.L.counts + 2) * ((P.D + 7) / 8)) {
            if (CHAINED) chain_wait();
            if (!fp_needed(p, q, s, it)) continue;        // uniform over the block
            const int etiles = (P.D + 7) / 8;             // near-axis rays: one per warp
            const int x = rem - fast_items;
            const int e = x / etiles;
            const int r = (x - e * etiles) * 8 + warp;
            if (r < P.D) {                                 // warp-uniform
                const int k = __ldg(q.L.exact + e);
                const float v = fp_exact_ray_warp(P, k, r, q.xpad + (size_t)s * np, q.xTpad + (size_t)s * np);
                if (lane == 0) e2 = residual(q, s, k, r, v);
            }
        } else {
            if (CHAINED) chain_wait();
            if (!fp_needed(p, q, s, it)) continue;        // uniform over the block
            // corner-clipping rays: one per warp
            const int gidx = (rem - fast_items - __ldg(q.L.counts + 2) * ((P.D + 7) / 8)) * 8 + warp;
            if (gidx < graze_count(q)) e2 = graze_ray(q, s, gidx);      // warp-uniform
        }
        e2acc += e2;
    }
    __syncthreads();
    flush_e2(it, cur, cur_slice, e2acc, sh);
}

// ---- phase BP of iteration `it` ------------------------------------------------
// One item: a tile of 32 columns x PIX*(8/bp_split) rows of slice s; thread
// (lane, warp) sums PIX rows of one column over its part of the angles.
// STAGED0: the caller already staged angle chunk 0 into sh.st.
template <int PIX, bool STAGED0>
__device__ __forceinline__ void bp_item(const SirtProblem &q, int s, int rem, SirtShared &sh) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const ProbGeom &P = q.P;
    const int SB = q.bp_split, lgSB = __ffs(SB) - 1, RB = 8 >> lgSB;   // angle parts, warp rows
    const int TR = PIX * RB;                         // tile rows
    const int tx_n = (P.N + 31) >> 5;
    const int ty = (int)((unsigned)rem / (unsigned)tx_n);
    const int tx = rem - ty * tx_n;
    const int wrow = warp >> lgSB, part = warp & (SB - 1);
    const size_t pr = (size_t)P.a * P.D, np = (size_t)P.N * (P.N + 2);
    const int col = tx * 32 + lane;
    const int row0 = ty * TR + wrow;
    const float xc = (float)(col - P.half) + 0.5f;
    const float yc0 = (float)(row0 - P.half) + 0.5f;
    const float *rr = q.rr + (size_t)s * pr;
    const bool unit = P.deltarho == 1.0f;
    const bool inrange = q.bp_inrange != 0;
    float sum[PIX], comp[PIX];
#pragma unroll
    for (int m = 0; m < PIX; ++m) sum[m] = comp[m] = 0.0f;
    for (int kc = 0; kc < P.a; kc += kBpChunk) {
        __syncthreads();
        if (!STAGED0 || kc > 0) bp_stage(P, kc, sh.st);
        __syncthreads();
        float prt[PIX];
#pragma unroll
        for (int m = 0; m < PIX; ++m) prt[m] = 0.0f;
        if (inrange) bp_chunk<PIX, true, true, true, 2>(P, sh.st, kc, P.a, part, SB, rr, xc, yc0, (float)RB, prt);
        else if (unit) bp_chunk<PIX, true, false, true, 2>(P, sh.st, kc, P.a, part, SB, rr, xc, yc0, (float)RB, prt);
        else bp_chunk<PIX, false, false, true>(P, sh.st, kc, P.a, part, SB, rr, xc, yc0, (float)RB, prt);
#pragma unroll
        for (int m = 0; m < PIX; ++m) comp_add(sum[m], comp[m], prt[m]);
    }
    float ex[PIX];
#pragma unroll
    for (int m = 0; m < PIX; ++m) ex[m] = 0.0f;
    bp_exact_angles<PIX>(P, q.L.exact, __ldg(q.L.counts + 2), part, SB, rr, row0, RB, col, ex);
#pragma unroll
    for (int m = 0; m < PIX; ++m) sh.red4[warp][m][lane] = (sum[m] + comp[m]) + ex[m];
    __syncthreads();
    float *xpad = q.xpad + (size_t)s * np;
    if (part == 0) {
#pragma unroll
        for (int m = 0; m < PIX; ++m) {
            float bpv = sh.red4[warp][m][lane];
            for (int t = 1; t < SB; ++t) bpv += sh.red4[warp + t][m][lane];
            const int row = row0 + RB * m;
            // the image corners add the terms of the rays that clip only
            // them (the warp of a corner row sums them; warp-uniform tests)
            if (row == 0 || row == P.N - 1) {
                const int cb = row == P.N - 1 ? 2 : 0;
                if (tx == 0) {
                    const float t = corner_terms_warp(q, s, cb);
                    if (col == 0) bpv = __fadd_rn(bpv, t);
                }
                if (tx == tx_n - 1) {
                    const float t = corner_terms_warp(q, s, cb + 1);
                    if (col == P.N - 1) bpv = __fadd_rn(bpv, t);
                }
            }
            float xi = 0.0f;
            if (row < P.N && col < P.N) {
                const size_t pix = (size_t)row * P.N + col;
                float *xp = xpad + (size_t)row * (P.N + 2) + col + 1;
                xi = __fadd_rn(*xp, __fmul_rn(q.C[pix], bpv));             // SIRT.fut:38-39
                *xp = xi;
            }
            sh.tile[lane][wrow + RB * m] = xi;
        }
    }
    __syncthreads();
    // transposed write: xTpad[col][row + 1] for the tile's 32 columns x TR rows
    float *xTpad = q.xTpad + (size_t)s * np;
    for (int i = threadIdx.x; i < 32 * TR; i += blockDim.x) {
        const int cl = i / TR, rl = i - cl * TR;
        const int c = tx * 32 + cl, r = ty * TR + rl;
        if (c < P.N && r < P.N) xTpad[(size_t)c * (P.N + 2) + r + 1] = sh.tile[cl][rl];
    }
}

template <bool CHAINED>
__device__ void bp_phase(const SirtParams &p, int it, unsigned *counter, SirtShared &sh) {
    const long long total = p.totals[1];
    for (long long item = next_item(p, counter, -1, sh); item < total; item = next_item(p, counter, item, sh)) {
        const int qi = find_problem(p, item, false);
        const SirtProblem &q = p.probs[qi];
        int s, rem;
        item_slice(item - q.bp_begin, q.bp_ips, s, rem);
        if (CHAINED) {
            // the first angle chunk's constants are static: stage them while
            // the forward phase finishes
            __syncthreads();
            bp_stage(q.P, 0, sh.st);
            chain_wait();
        }
        if (!bp_needed(p, q, s, it)) continue;            // uniform over the block
        switch (q.bp_pix) {                               // uniform over the block
            case 1: bp_item<1, CHAINED>(q, s, rem, sh); break;
            case 2: bp_item<2, CHAINED>(q, s, rem, sh); break;
            default: bp_item<4, CHAINED>(q, s, rem, sh); break;
        }
    }
}

__global__ void __launch_bounds__(256, 3) sirt_persistent_kernel(SirtParams p) {
    __shared__ SirtShared sh;
    const unsigned nb = gridDim.x + p.barrier_extra;
    for (int it = 0; it <= p.max_iterations; ++it) {
        // phase 2*it: FP.  Rotating counters: reset the one of the phase after next.
        const int ph = 2 * it;
        if (p.dynamic && blockIdx.x == 0 && threadIdx.x == 0) p.work[(ph + 1) % 3] = 0u;
        fp_phase<false>(p, it, p.work + ph % 3, sh);
        if (!grid_barrier(p.bar, nb, p.status, p.timeout_ns, &sh.flag)) return;
        if (it == p.max_iterations) break;
        // stopping rule (identical decision in every block)
        if (p.tol2 > 0.0) {
            if (threadIdx.x == 0) sh.any = 0;
            __syncthreads();
            for (int qi = 0; qi < p.nprob; ++qi) {
                const SirtProblem &q = p.probs[qi];
                for (int s = threadIdx.x; s < q.nslices; s += blockDim.x) {
                    if (bp_needed(p, q, s, it)) sh.any = 1;
                    else if (blockIdx.x == 0 && it < q.iterations && stop_of(q, s) > it) q.stop_iter[s] = it;
                }
            }
            __syncthreads();
            if (!sh.any) break;
        }
        const int ph2 = ph + 1;
        if (p.dynamic && blockIdx.x == 0 && threadIdx.x == 0) p.work[(ph2 + 1) % 3] = 0u;
        bp_phase<false>(p, it, p.work + ph2 % 3, sh);
        if (!grid_barrier(p.bar, nb, p.status, p.timeout_ns, &sh.flag)) return;
    }
}


// Phase-split engine: the same two phases as ordinary launches, one per phase
// and iteration.  The kernel boundary replaces the grid barrier, which for
// small iterations (a few slices of N <= 256) is cheaper than the persistent
// kernel's two barriers per iteration; each kernel also gets its own register
// allocation.  Items are assigned statically (item = block + i*grid).
__global__ void __launch_bounds__(256, 5) sirt_fp_phase_kernel(SirtParams p, int it) {
    __shared__ SirtShared sh;
    chain_release();
    fp_phase<true>(p, it, nullptr, sh);
    chain_wait();                        // blocks without items wait too
}

// Forward phase of the split engine for a single problem (a stack of slices):
// the standalone projector's grid (8/S detectors x S row parts per block, one
// angle group per blockIdx.y, one slice per blockIdx.z) with the residual as
// its epilogue.  Without the phase functions' item bookkeeping it keeps the
// projector's register count and occupancy; the per-ray values are those of
// fp_phase (same rows, same split, same order), so the iterates are the same.
template <int S>
__global__ void __launch_bounds__(256) sirt_fp_stack_kernel(SirtProblem q, int it, double tol2, int record_final) {
    __shared__ float red[8][32];
    __shared__ double e2s;
    const int s = blockIdx.z;
    if (it > q.iterations || (it == q.iterations && !record_final)) return;       // block-uniform
    if (tol2 > 0.0 && stop_of(q, s) < it) return;
    const int grp = blockIdx.y;
    const int nsteep = __ldg(q.L.counts), nflat = __ldg(q.L.counts + 1);
    if (grp >= nsteep + nflat) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) e2s = 0.0;
    const int part = warp % S;
    // S = 1: 4 angles x 8 detectors per warp, as the standalone projector
    // (N=512 / 360 angles stack: 117 -> 108 us per slice-iteration)
    const int r = S == 1 ? blockIdx.x * 8 + (lane & 7) : blockIdx.x * (8 / S) + warp / S;
    const int rr = r < q.P.D ? r : q.P.D - 1;
    const int k = __ldg(q.L.order + grp * 32 + (S == 1 ? warp * 4 + (lane >> 3) : lane));
    const int jb = (int)((long long)part * q.P.N / S), je = (int)((long long)(part + 1) * q.P.N / S);
    const size_t np = (size_t)q.P.N * (q.P.N + 2);
    const float *img = (grp < nsteep ? q.xpad : q.xTpad) + (size_t)s * np;
    const int kk = r < q.P.D ? k : -1;
    const float v = fp_lane_ray(q.P, kk, rr, img, jb, je);
    red[warp][lane] = v;
    __syncthreads();
    double e2 = 0.0;
    if (part == 0 && kk >= 0) {
        float fpv = red[warp][lane];
        for (int t = 1; t < S; ++t) fpv += red[warp + t][lane];
        e2 = residual(q, s, kk, r, fpv);
    }
    e2 = warp_sum_d(e2);
    if (lane == 0 && e2 != 0.0) atomicAdd(&e2s, e2);
    __syncthreads();
    if (threadIdx.x == 0 && e2s != 0.0) atomicAdd(q.res2 + (size_t)s * (q.iterations + 1) + it, e2s);
}

// Near-axis rays of the same phase: a warp per ray (8 detectors per block),
// kExactSlotsSirt angle slots, one slice per blockIdx.z.
constexpr int kExactSlotsSirt = 4;

__global__ void __launch_bounds__(256) sirt_fp_stack_exact_kernel(SirtProblem q, int it, double tol2,
                                                                  int record_final) {
    __shared__ double e2s;
    const int s = blockIdx.z;
    if (it > q.iterations || (it == q.iterations && !record_final)) return;
    if (tol2 > 0.0 && stop_of(q, s) < it) return;
    const int nexact = __ldg(q.L.counts + 2);
    const int ngraze = graze_count(q);
    // blocks of slot row 0 also walk the corner-clipping rays, one per warp
    if ((int)blockIdx.y >= nexact && (blockIdx.y != 0 || ngraze == 0)) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (threadIdx.x == 0) e2s = 0.0;
    __syncthreads();
    const int r = blockIdx.x * 8 + warp;
    const size_t np = (size_t)q.P.N * (q.P.N + 2);
    double e2 = 0.0;
    for (int e = blockIdx.y; e < nexact; e += gridDim.y) {
        const int k = __ldg(q.L.exact + e);
        if (r < q.P.D) {                                   // warp-uniform
            const float v = fp_exact_ray_warp(q.P, k, r, q.xpad + (size_t)s * np, q.xTpad + (size_t)s * np);
            if (lane == 0) e2 += residual(q, s, k, r, v);
        }
    }
    if (blockIdx.y == 0)
        for (int gidx = blockIdx.x * 8 + warp; gidx < ngraze; gidx += gridDim.x * 8) e2 += graze_ray(q, s, gidx);
    if (lane == 0 && e2 != 0.0) atomicAdd(&e2s, e2);
    __syncthreads();
    if (threadIdx.x == 0 && e2s != 0.0) atomicAdd(q.res2 + (size_t)s * (q.iterations + 1) + it, e2s);
}

// Block 0 also applies the stopping rule of iteration it (the same decision
// as the fused kernel: every block's bp_needed reads the same residuals) and
// stores the number of slices still updating in *active.
__global__ void __launch_bounds__(256, 4) sirt_bp_phase_kernel(SirtParams p, int it, int *active) {
    __shared__ SirtShared sh;
    chain_release();
    if (blockIdx.x == 0) {
        chain_wait();                    // the stopping rule reads the forward phase's residuals
        if (threadIdx.x == 0) sh.any = 0;
        __syncthreads();
        int cnt = 0;
        for (int qi = 0; qi < p.nprob; ++qi) {
            const SirtProblem &q = p.probs[qi];
            for (int s = threadIdx.x; s < q.nslices; s += blockDim.x) {
                if (bp_needed(p, q, s, it)) ++cnt;
                else if (p.tol2 > 0.0 && it < q.iterations && stop_of(q, s) > it) q.stop_iter[s] = it;
            }
        }
        if (cnt) atomicAdd(&sh.any, cnt);
        __syncthreads();
        if (threadIdx.x == 0) *active = sh.any;
    }
    bp_phase<true>(p, it, nullptr, sh);
    chain_wait();                        // blocks without items wait too
}

// Backward phase of the split engine for one large problem (a slice stack)
// on the standalone backprojector's grid: a block = 32 columns x 64 rows of
// one slice (blockIdx.z), 8 rows per thread, the weighted residual read as
// detector pairs (one 8-byte gather per pixel and angle), four angles at a
// time, and the SIRT update x + C*bp (SIRT.fut:38-39) with both padded
// copies of the iterate in the epilogue.  The angles are summed in the order
// of bp_phase; a pixel's detector coordinate comes from its thread's first
// row, so the iterates equal the generic phase's to rounding.  Block (0,0,0)
// also applies the stopping rule of iteration it (sirt_bp_phase_kernel's rule).
__global__ void __launch_bounds__(256, 4) sirt_bp_stack_kernel(SirtProblem q, int it, double tol2, int *active) {
    __shared__ BpStage st;
    __shared__ float tile[32][65];
    __shared__ int any;
    const int s = blockIdx.z;
    if (blockIdx.x == 0 && blockIdx.y == 0 && blockIdx.z == 0) {
        if (threadIdx.x == 0) any = 0;
        __syncthreads();
        int cnt = 0;
        for (int z = threadIdx.x; z < q.nslices; z += blockDim.x) {
            if (bp_needed(tol2, q, z, it)) ++cnt;
            else if (tol2 > 0.0 && it < q.iterations && stop_of(q, z) > it) q.stop_iter[z] = it;
        }
        if (cnt) atomicAdd(&any, cnt);
        __syncthreads();
        if (threadIdx.x == 0) *active = any;
    }
    if (!bp_needed(tol2, q, s, it)) return;              // block-uniform
    const ProbGeom &P = q.P;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int col = blockIdx.x * 32 + lane;
    const int row0 = blockIdx.y * 64 + warp;
    const float xc = (float)(col - P.half) + 0.5f;
    const float yc0 = (float)(row0 - P.half) + 0.5f;
    const size_t pr = (size_t)P.a * P.D, np = (size_t)P.N * (P.N + 2);
    const float *rows = q.rrp + (size_t)s * pr * 2;
    float sum[8], comp[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) sum[m] = comp[m] = 0.0f;
    for (int kc = 0; kc < P.a; kc += kBpChunk) {
        __syncthreads();
        bp_stage(P, kc, st);
        __syncthreads();
        float part[8];
#pragma unroll
        for (int m = 0; m < 8; ++m) part[m] = 0.0f;
        bp_chunk<8, true, true, true, 4, true>(P, st, kc, P.a, 0, 1, rows, xc, yc0, 8.0f, part);
#pragma unroll
        for (int m = 0; m < 8; ++m) comp_add(sum[m], comp[m], part[m]);
    }
    float ex[8];
#pragma unroll
    for (int m = 0; m < 8; ++m) ex[m] = 0.0f;
    bp_exact_angles<8>(P, q.L.exact, __ldg(q.L.counts + 2), 0, 1, q.rr + (size_t)s * pr, row0, 8, col, ex);
    float *xpad = q.xpad + (size_t)s * np;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
        float bpv = (sum[m] + comp[m]) + ex[m];
        const int row = row0 + 8 * m;
        // the image corners add the terms of the rays that clip only them
        // (warp-uniform tests: the warp of a corner row sums them)
        if (row == 0 || row == P.N - 1) {
            const int cb = row == P.N - 1 ? 2 : 0;
            if (blockIdx.x == 0) {
                const float t = corner_terms_warp(q, s, cb);
                if (col == 0) bpv = __fadd_rn(bpv, t);
            }
            if (blockIdx.x == gridDim.x - 1) {
                const float t = corner_terms_warp(q, s, cb + 1);
                if (col == P.N - 1) bpv = __fadd_rn(bpv, t);
            }
        }
        float xi = 0.0f;
        if (row < P.N && col < P.N) {
            float *xp = xpad + (size_t)row * (P.N + 2) + col + 1;
            xi = __fadd_rn(*xp, __fmul_rn(q.C[(size_t)row * P.N + col], bpv));      // SIRT.fut:38-39
            *xp = xi;
        }
        tile[lane][warp + 8 * m] = xi;
    }
    __syncthreads();
    // transposed write: xTpad[col][row + 1] for the tile's 32 columns x 64 rows
    float *xTpad = q.xTpad + (size_t)s * np;
    for (int i = threadIdx.x; i < 32 * 64; i += blockDim.x) {
        const int cl = i >> 6, rl = i & 63;
        const int c = blockIdx.x * 32 + cl, r = blockIdx.y * 64 + rl;
        if (c < P.N && r < P.N) xTpad[(size_t)c * (P.N + 2) + r + 1] = tile[cl][rl];
    }
}

cudaError_t launch_sirt_bp_stack(const SirtProblem &q, int it, double tol2, int *active, cudaStream_t stream) {
    const dim3 grid((q.P.N + 31) / 32, (q.P.N + 63) / 64, q.nslices);
    sirt_bp_stack_kernel<<<grid, 256, 0, stream>>>(q, it, tol2, active);
    return cudaGetLastError();
}

// Per-problem item counts and begin offsets (depend on the angle lists).
__global__ void sirt_plan_kernel(SirtProblem *probs, int nprob, long long *totals) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    long long fb = 0, bb = 0;
    for (int i = 0; i < nprob; ++i) {
        SirtProblem &q = probs[i];
        const int G = 8 / q.fp_split;
        const int ngroups = q.L.counts[0] + q.L.counts[1];
        const int nexact = q.L.counts[2];
        q.fp_ips = ngroups * ((q.P.D + G - 1) / G) + nexact * ((q.P.D + 7) / 8) + (q.goff[4] + 7) / 8;
        const int TR = q.bp_pix * (8 / q.bp_split);
        q.bp_ips = ((q.P.N + 31) / 32) * ((q.P.N + TR - 1) / TR);
        q.fp_begin = fb;
        q.bp_begin = bb;
        fb += (long long)q.fp_ips * q.nslices;
        bb += (long long)q.bp_ips * q.nslices;
    }
    totals[0] = fb;
    totals[1] = bb;
}

cudaError_t launch_sirt_plan(SirtProblem *probs, int nprob, long long *totals, cudaStream_t stream) {
    sirt_plan_kernel<<<1, 32, 0, stream>>>(probs, nprob, totals);
    return cudaGetLastError();
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

cudaError_t launch_sumsq(const float *b, size_t len, int nslices, double *out, cudaStream_t stream) {
    dim3 grid(64, nslices);
    sumsq_kernel<<<grid, 256, 0, stream>>>(b, len, out);
    return cudaGetLastError();
}

// residuals[s][k] = sqrt(res2[s][k] / b2[s]); iterations_done[s].
__global__ void sirt_finalize_kernel(SirtProblem *probs, int record_final) {
    const SirtProblem &q = probs[blockIdx.y];
    const int s = blockIdx.x;
    if (s >= q.nslices) return;
    const int K = q.iterations + 1;
    const int stop = q.stop_iter[s] < q.iterations ? q.stop_iter[s] : q.iterations;
    if (threadIdx.x == 0 && q.iters_done) q.iters_done[s] = stop;
    if (!q.residuals) return;
    const int last = record_final ? q.iterations : q.iterations - 1;
    for (int k = threadIdx.x; k < K; k += blockDim.x) {
        if (k > stop || k > last) continue;
        const double b2 = q.b2[s];
        q.residuals[(size_t)s * K + k] = b2 > 0.0 ? sqrt(q.res2[(size_t)s * K + k] / b2) : 0.0;
    }
}

cudaError_t launch_sirt_finalize(SirtProblem *probs, int nprob, int max_slices, int record_final,
                                 cudaStream_t stream) {
    dim3 grid(max_slices, nprob);
    sirt_finalize_kernel<<<grid, 128, 0, stream>>>(probs, record_final);
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

int sirt_phase_grids(int *fp_grid, int *bp_grid) {
    int dev = 0, sms = 0, f = 0, b = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f, sirt_fp_phase_kernel, 256, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, sirt_bp_phase_kernel, 256, 0);
    *fp_grid = sms * f;
    *bp_grid = sms * b;
    return f > 0 && b > 0;
}

// A launch of 256-thread blocks that may begin while the previous kernel in
// the stream finishes (programmatic stream serialization; the kernel waits).
template <class... KArgs, class... Args>
static cudaError_t launch_chained(void (*kernel)(KArgs...), int grid, cudaStream_t stream, Args... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, args...);
}

cudaError_t launch_sirt_fp_phase(const SirtParams &p, int it, int grid, cudaStream_t stream) {
    return launch_chained(sirt_fp_phase_kernel, grid, stream, p, it);
}

cudaError_t launch_sirt_fp_stack(const SirtProblem &q, int it, double tol2, int record_final, cudaStream_t stream) {
    const int S = q.fp_split;
    const int gmax = (q.P.a + 31) / 32 + 2;
    const dim3 grid((q.P.D + 8 / S - 1) / (8 / S), gmax, q.nslices);
    switch (S) {
        case 1: sirt_fp_stack_kernel<1><<<grid, 256, 0, stream>>>(q, it, tol2, record_final); break;
        case 2: sirt_fp_stack_kernel<2><<<grid, 256, 0, stream>>>(q, it, tol2, record_final); break;
        case 4: sirt_fp_stack_kernel<4><<<grid, 256, 0, stream>>>(q, it, tol2, record_final); break;
        default: sirt_fp_stack_kernel<8><<<grid, 256, 0, stream>>>(q, it, tol2, record_final); break;
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    const dim3 ge((q.P.D + 7) / 8, kExactSlotsSirt, q.nslices);
    sirt_fp_stack_exact_kernel<<<ge, 256, 0, stream>>>(q, it, tol2, record_final);
    return cudaGetLastError();
}

cudaError_t launch_sirt_bp_phase(const SirtParams &p, int it, int *active, int grid, cudaStream_t stream) {
    return launch_chained(sirt_bp_phase_kernel, grid, stream, p, it, active);
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

}  // namespace synk

// batch_impl.cuh -- many independent layouts in one persistent launch.
// Included by inst_f32.cu and inst_f64.cu only.
//
// Each graph of a batch is laid out by one thread block from start to end:
// the block takes the next graph from a work counter (largest first), then
// runs every step of every requested iteration for it:
//   - bounding box;
//   - Morton codes;
//   - a block-level stable radix sort;
//   - the Karras tree;
//   - the bottom-up sums with block-scope arrivals;
//   - the Barnes-Hut walk (or the exact all-pairs sum below the crossover);
//   - gravity and attraction;
//   - the swing/traction totals reduced by the block, the FP64 speed update
//     of that graph;
//   - the displacement.
// No block ever waits for another, and a graph's result depends on nothing
// but the graph and the block size: it is the same alone or in any mix.
//
// Device arrays are the concatenation of the graphs' arrays (node arrays at
// the graph's first node, its incidences at its first incidence, node indices
// of the incidences local to the graph); the tree arrays of a graph of n
// nodes use n (or 2n for parent) entries from its first node (2x for parent).
#pragma once

#include <algorithm>
#include <cmath>
#include <map>
#include <numeric>
#include <string.h>
#include <vector>

#include "karras.cuh"
#include "kernels.cuh"
#include "layout_impl.cuh" // DevMem
#include "session.h"

namespace fa2cu {

// One graph of a batch, in device memory; the speed state is updated by the
// block that lays the graph out.
struct BatchGraph {
    int n;      // nodes
    int node0;  // first node in the concatenated node arrays
    int exact;  // 1: all-pairs repulsion, 0: Barnes-Hut
    int flags;  // bit 0 strong, 1 linlog, 2 adjust, 3 some node fixed
    double scaling, gravity, theta2d, jitter;
    double speed, efficiency, total_swinging, total_traction;
    int err, pad;
};

// BF_HUBS: a node of mass HUB_MASS or more (FP32: the walk compensates its
// sums)
enum { BF_STRONG = 1, BF_LINLOG = 2, BF_ADJUST = 4, BF_FIXED = 8, BF_HUBS = 16 };

template <class R> struct BatchArrays {
    typedef typename RT<R>::R2 R2;
    typedef typename RT<R>::R4 R4;
    R2 *pos, *f, *fold;
    R *mass, *size, *sw, *tr;
    uint8_t *fixed;
    int *off; // incidence range of node i: off[i] .. off[i+1]-1 (global)
    Inc<R> *inc;
    uint32_t *key, *idx, *key_b, *idx_b;
    R4 *psort;
    int2 *child, *range;
    int *parent, *rope, *visits;
    Agg<R> *agg;
    R4 *rec_c;  // traversal records (common.cuh)
    int2 *rec_t;
    // per block, the cycles spent in each of the 8 phases of an iteration
    // (measurement launches only; nullptr otherwise)
    unsigned long long *prof;
};

// Phases of a batched iteration, as counted in BatchArrays::prof.
enum { BP_CODES, BP_SORT, BP_TREE, BP_SUMS, BP_REPULSION, BP_ATTRACTION, BP_TOTALS, BP_MOVE };

// ---- block-level building blocks ----------------------------------------------

// (block_sort_pairs, the one-block radix sort, is in sort_tree.cuh)

// Sum over the block in a fixed order (per thread, per warp by shuffles, over
// the warps by thread 0); the result is valid in thread 0.
template <int W> __device__ double block_sum(double v, double *scratch)
{
    v = warp_sum(v);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    __syncthreads();
    if (lane == 0) scratch[w] = v;
    __syncthreads();
    double s = 0.0, c = 0.0;
    if (threadIdx.x == 0)
        for (int k = 0; k < W; k++) neumaier(s, c, scratch[k]);
    return __dadd_rn(s, c);
}

// ---- the persistent kernel -----------------------------------------------------

// FP32: three blocks of 512 (six of 256) threads per SM, 40 registers a
// thread (~120 bytes of spills, in the sort and tree phases): 48 warps
// resident for the walk, which is bound by instruction issue. Against two
// blocks of 512 at 63 registers: 7.30 -> 6.49 ms a batch iteration of 4096
// graphs; four blocks (32 registers, ~400 bytes of spills) 6.60-6.70 ms.
// FP64 needs more registers: one block of 512 (two of 256).
template <class R, int T>
__global__ void __launch_bounds__(T, (sizeof(R) == 8 ? 512 : 1536) / T)
k_batch(int ngraphs, BatchGraph *graphs, const int *queue, int *next, int iterations,
        BatchArrays<R> A, int npt, int *status)
{
    typedef typename RT<R>::R2 R2;
    typedef typename RT<R>::R4 R4;
    constexpr int W = T / 32;
    // the sort's digit counts; the exact sum's record tile (T records of at
    // most 32 bytes) in the same space
    __shared__ __align__(16) uint32_t cnt[W][256];
    __shared__ uint32_t dbase[256];
    __shared__ double red[W], red2[W];
    __shared__ R mins[4][W];
    __shared__ double quant[3];
    __shared__ double sh_speed;
    __shared__ int sh_g, sh_stop;
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;

    for (;;) {
        if (tid == 0) sh_g = atomicAdd(next, 1);
        __syncthreads();
        const int qi = sh_g;
        __syncthreads();
        if (qi >= ngraphs) break;
        BatchGraph *G = graphs + queue[qi];
        const int n = G->n, b0 = G->node0;
        const bool exact = G->exact != 0;
        const int flags = G->flags;
        const bool strong = flags & BF_STRONG, linlog = flags & BF_LINLOG;
        const bool adjust = flags & BF_ADJUST, anyfix = flags & BF_FIXED;
        const bool hubs = flags & BF_HUBS;
        const R scaling = (R) G->scaling, gravity = (R) G->gravity;
        const double theta2d = G->theta2d;
        const R theta2 = (R) theta2d;
        // the FP32 records' scale of size^2 (region_far)
        const R wscale = (R) ((1.0 + (double) DECIDE_BAND) / theta2d);
        R2 *pos = A.pos + b0, *f = A.f + b0, *fold = A.fold + b0;
        const R *mass = A.mass + b0;
        const R *size = A.size ? A.size + b0 : nullptr;
        R *sw = A.sw + b0, *tr = A.tr ? A.tr + b0 : nullptr;
        const uint8_t *fixed = anyfix ? A.fixed + b0 : nullptr;
        const int *off = A.off + b0;
        uint32_t *key = A.key + b0, *idx = A.idx + b0, *kb = A.key_b + b0, *vb = A.idx_b + b0;
        R4 *psort = A.psort + b0;
        int2 *child = A.child + b0, *range = A.range + b0;
        int *parent = A.parent + 2 * (size_t) b0, *rope = A.rope + b0, *visits = A.visits + b0;
        Agg<R> *agg = A.agg + b0;
        R4 *rec_c = A.rec_c + b0;
        int2 *rec_t = A.rec_t + b0;
        if (tid == 0) {
            sh_speed = G->speed;
            sh_stop = 0;
        }
        double speed = G->speed, eff = G->efficiency;

        // phase clock of thread 0, read after each block-wide barrier
        long long tlast = clock64();
        auto phase = [&](int ph) {
            if (A.prof && tid == 0) {
                const long long t = clock64();
                A.prof[(size_t) blockIdx.x * 8 + ph] += (unsigned long long) (t - tlast);
                tlast = t;
            }
        };
        for (int it = 0; it < iterations; it++) {
            __syncthreads();
            phase(BP_MOVE);
            if (sh_stop) break;
            if (exact || n < 2) {
                // records in original order; the all-pairs sum per node over
                // tiles of T records staged in shared memory (in node order)
                for (int i = tid; i < n; i += T) {
                    const R2 p = pos[i];
                    psort[i] = mk4<R>(p.x, p.y, mass[i], adjust ? size[i] : R(0));
                }
                R4 *tile = reinterpret_cast<R4 *>(&cnt[0][0]);
                // the tile shape (autotuned): npt = 2 nodes per thread (i
                // and i + T), each tile record feeding two independent sums,
                // or 1; every node sums j ascending either way
                const bool two = npt == 2 && n > T;
                for (int i0 = 0; i0 < n; i0 += two ? 2 * T : T) {
                    const int ia = i0 + tid, ib = two ? ia + T : n;
                    const R4 zero = mk4<R>(R(0), R(0), R(0), R(0));
                    const R4 ma = ia < n ? psort[ia] : zero, mb = ib < n ? psort[ib] : zero;
                    R axa = R(0), aya = R(0), axb = R(0), ayb = R(0);
                    const float smia = (float) scaling * (float) ma.z;
                    const float smib = (float) scaling * (float) mb.z;
                    for (int j0 = 0; j0 < n; j0 += T) {
                        __syncthreads();
                        if (j0 + tid < n) tile[tid] = psort[j0 + tid];
                        __syncthreads();
                        const int m = min(T, n - j0);
                        if (sizeof(R) == 4 && !adjust) {
                            // d2 carries 1e-30 (as k_exact): a coincident
                            // pair (xd = yd = 0) has a finite factor, so it
                            // adds 0, the reference's factor for d2 = 0
                            if (!two) { // one node per thread
#pragma unroll 4
                                for (int jj = 0; jj < m; jj++) {
                                    const R4 q = tile[jj];
                                    const float xda = (float) ma.x - (float) q.x;
                                    const float yda = (float) ma.y - (float) q.y;
                                    const float d2a = fmaf(xda, xda, fmaf(yda, yda, 1e-30f));
                                    const float ga = (float) q.z * __fdividef(1.0f, d2a);
                                    axa = (R) fmaf(xda, ga, (float) axa);
                                    aya = (R) fmaf(yda, ga, (float) aya);
                                }
                            } else {
#pragma unroll 4
                                for (int jj = 0; jj < m; jj++) {
                                    const R4 q = tile[jj];
                                    const float xda = (float) ma.x - (float) q.x;
                                    const float yda = (float) ma.y - (float) q.y;
                                    const float xdb = (float) mb.x - (float) q.x;
                                    const float ydb = (float) mb.y - (float) q.y;
                                    const float d2a = fmaf(xda, xda, fmaf(yda, yda, 1e-30f));
                                    const float d2b = fmaf(xdb, xdb, fmaf(ydb, ydb, 1e-30f));
                                    const float ga = (float) q.z * __fdividef(1.0f, d2a);
                                    const float gb = (float) q.z * __fdividef(1.0f, d2b);
                                    axa = (R) fmaf(xda, ga, (float) axa);
                                    aya = (R) fmaf(yda, ga, (float) aya);
                                    axb = (R) fmaf(xdb, gb, (float) axb);
                                    ayb = (R) fmaf(ydb, gb, (float) ayb);
                                }
                            }
                        } else {
                            for (int jj = 0; jj < m; jj++) {
                                const R4 q = tile[jj];
                                const R xda = ma.x - q.x, yda = ma.y - q.y;
                                const R xdb = mb.x - q.x, ydb = mb.y - q.y;
                                R ga, gb;
                                if (adjust) {
                                    ga = rep_factor<R, true>(xda * xda + yda * yda, ma.z * q.z,
                                                             ma.w + q.w, scaling);
                                    gb = rep_factor<R, true>(xdb * xdb + ydb * ydb, mb.z * q.z,
                                                             mb.w + q.w, scaling);
                                } else {
                                    ga = rep_factor<R, false>(xda * xda + yda * yda, ma.z * q.z,
                                                              R(0), scaling);
                                    gb = rep_factor<R, false>(xdb * xdb + ydb * ydb, mb.z * q.z,
                                                              R(0), scaling);
                                }
                                axa += xda * ga;
                                aya += yda * ga;
                                axb += xdb * gb;
                                ayb += ydb * gb;
                            }
                        }
                    }
                    if (sizeof(R) == 4 && !adjust) { // scaling * m_i, once
                        axa = (R) ((float) axa * smia);
                        aya = (R) ((float) aya * smia);
                        axb = (R) ((float) axb * smib);
                        ayb = (R) ((float) ayb * smib);
                    }
                    if (ia < n) f[ia] = mk2<R>(axa, aya);
                    if (ib < n) f[ib] = mk2<R>(axb, ayb);
                }
            } else {
                // bounding box and the Morton quantisation
                R mnx = pos[0].x, mxx = mnx, mny = pos[0].y, mxy = mny;
                for (int i = tid; i < n; i += T) {
                    const R2 p = pos[i];
                    mnx = cl_min(mnx, p.x);
                    mny = cl_min(mny, p.y);
                    mxx = cl_max(mxx, p.x);
                    mxy = cl_max(mxy, p.y);
                }
                for (int o = 16; o > 0; o >>= 1) {
                    mnx = cl_min(mnx, __shfl_down_sync(0xffffffffu, mnx, o));
                    mny = cl_min(mny, __shfl_down_sync(0xffffffffu, mny, o));
                    mxx = cl_max(mxx, __shfl_down_sync(0xffffffffu, mxx, o));
                    mxy = cl_max(mxy, __shfl_down_sync(0xffffffffu, mxy, o));
                }
                if (lane == 0) {
                    mins[0][w] = mnx;
                    mins[1][w] = mny;
                    mins[2][w] = mxx;
                    mins[3][w] = mxy;
                }
                __syncthreads();
                if (tid == 0) {
                    for (int k = 1; k < W; k++) {
                        mnx = cl_min(mnx, mins[0][k]);
                        mny = cl_min(mny, mins[1][k]);
                        mxx = cl_max(mxx, mins[2][k]);
                        mxy = cl_max(mxy, mins[3][k]);
                    }
                    const double wd = __dsub_rn((double) mxx, (double) mnx);
                    const double hd = __dsub_rn((double) mxy, (double) mny);
                    const double ext = cl_max(wd, hd);
                    quant[0] = (double) mnx;
                    quant[1] = (double) mny;
                    quant[2] = ext > 0.0 ? __ddiv_rn(65535.0, ext) : 0.0;
                }
                __syncthreads();
                for (int i = tid; i < n; i += T) {
                    const R2 p = pos[i];
                    const double fx = cl_min(
                        cl_max(__dmul_rn(__dsub_rn((double) p.x, quant[0]), quant[2]), 0.0),
                        65535.0);
                    const double fy = cl_min(
                        cl_max(__dmul_rn(__dsub_rn((double) p.y, quant[1]), quant[2]), 0.0),
                        65535.0);
                    key[i] = spread16((uint32_t) fx) | (spread16((uint32_t) fy) << 1);
                    idx[i] = (uint32_t) i;
                }
                __syncthreads();
                phase(BP_CODES);
                block_sort_pairs<W>(n, key, idx, kb, vb, cnt, dbase);
                phase(BP_SORT);
                for (int k = tid; k < n; k += T) {
                    const uint32_t i = idx[k];
                    const R2 p = pos[i];
                    psort[k] = mk4<R>(p.x, p.y, mass[i], adjust ? size[i] : R(0));
                }
                for (int i = tid; i < n - 1; i += T)
                    karras_one<false>(i, n, key, child, range, parent, rope, visits);
                __syncthreads();
                phase(BP_TREE);
                // contiguous leaves per thread: a thread's later climbs find
                // the regions of its earlier ones complete
                const int per = (n + T - 1) / T;
                for (int q = 0; q < per; q++) {
                    const int k = tid * per + q;
                    if (k < n)
                        climb<R, true>(k, n, psort, child, parent, range, rope, visits, agg,
                                       rec_c, rec_t, wscale, status);
                }
                __syncthreads();
                phase(BP_SUMS);
                // FP32: the walk with its node pairs deferred (the single
                // layout's), compensated for hubs; FP64: the per-thread walk
                // in the reference's order
                for (int k = tid; k < n; k += T) {
                    R2 fk;
                    if constexpr (sizeof(R) == 4) {
                        if (hubs)
                            fk = adjust ? walk_deferred<R, true, true>(k, n, scaling, theta2,
                                                                       theta2d, psort, rec_c,
                                                                       rec_t, agg, rope, status)
                                        : walk_deferred<R, false, true>(k, n, scaling, theta2,
                                                                        theta2d, psort, rec_c,
                                                                        rec_t, agg, rope, status);
                        else
                            fk = adjust ? walk_deferred<R, true>(k, n, scaling, theta2, theta2d,
                                                                 psort, rec_c, rec_t, agg, rope,
                                                                 status)
                                        : walk_deferred<R, false>(k, n, scaling, theta2, theta2d,
                                                                  psort, rec_c, rec_t, agg, rope,
                                                                  status);
                    } else {
                        fk = adjust ? walk<R, true>(k, n, scaling, theta2, theta2d, psort, rec_c,
                                                    rec_t, agg, rope, status)
                                    : walk<R, false>(k, n, scaling, theta2, theta2d, psort, rec_c,
                                                     rec_t, agg, rope, status);
                    }
                    f[idx[k]] = fk;
                }
            }
            __syncthreads();
            phase(BP_REPULSION);
            for (int i = tid; i < n; i += T)
                attract_one<R>(i, gravity, strong, linlog, adjust, pos, mass, size, off, A.inc,
                               f);
            __syncthreads();
            phase(BP_ATTRACTION);
            // swinging and traction; totals in double in a fixed order: in
            // FP64 up to SERIAL_TOTALS_MAX nodes serially in node order (the
            // reference's order, as the single-graph path), else per thread
            // and over the block
            const bool serial = serial_totals<R>(n);
            double ts = 0.0, tt = 0.0;
            for (int i = tid; i < n; i += T) {
                const R2 a = f[i], b = fold[i];
                const R sx = b.x - a.x, sy = b.y - a.y;
                const R tx = b.x + a.x, ty = b.y + a.y;
                const R m = mass[i];
                const R s = m * fsqrt(sx * sx + sy * sy);
                const R t = R(0.5) * m * fsqrt(tx * tx + ty * ty);
                sw[i] = s;
                if (serial) tr[i] = t;
                if (fixed && fixed[i]) continue;
                ts = __dadd_rn(ts, (double) s);
                tt = __dadd_rn(tt, (double) t);
            }
            double tsw = block_sum<W>(ts, red);
            double ttr = block_sum<W>(tt, red2);
            if (serial) {
                __syncthreads(); // sw / tr written by every thread
                if (tid == 0) {
                    tsw = 0.0;
                    ttr = 0.0;
                    for (int i = 0; i < n; i++) {
                        if (fixed && fixed[i]) continue;
                        tsw = __dadd_rn(tsw, (double) sw[i]);
                        ttr = __dadd_rn(ttr, (double) tr[i]);
                    }
                }
            }
            if (tid == 0) {
                if (!(tsw == tsw) || !(ttr == ttr)) {
                    sh_stop = 1;
                    G->err = ERR_NAN;
                    atomicOr(status + ST_ERROR, ERR_NAN);
                } else {
                    SpeedState s0;
                    s0.speed = speed;
                    s0.efficiency = eff;
                    s0.n = n;
                    s0.jitter_tolerance = G->jitter;
                    update_speed_dev(&s0, tsw, ttr);
                    speed = s0.speed;
                    eff = s0.efficiency;
                    sh_speed = speed;
                    G->total_swinging = tsw;
                    G->total_traction = ttr;
                }
            }
            __syncthreads();
            phase(BP_TOTALS);
            if (sh_stop) break;
            const R sp = (R) sh_speed;
            for (int i = tid; i < n; i += T) {
                const R2 a = f[i];
                fold[i] = a;
                if (fixed && fixed[i]) continue;
                R factor;
                if (adjust) {
                    const R df = fsqrt(a.x * a.x + a.y * a.y);
                    factor = fdiv(R(0.1) * sp, R(1) + fsqrt(sp * sw[i]));
                    if (df > R(0)) {
                        if (factor * df > R(10)) factor = fdiv(R(10), df);
                    } else {
                        factor = R(0);
                    }
                } else {
                    factor = fdiv(sp, R(1) + fsqrt(sp * sw[i]));
                }
                R2 p = pos[i];
                p.x += a.x * factor;
                p.y += a.y * factor;
                pos[i] = p;
            }
        }
        __syncthreads();
        if (tid == 0) {
            G->speed = speed;
            G->efficiency = eff;
        }
    }
}

// ---- host side -------------------------------------------------------------------

template <class R> struct Batch : BatchBase {
    typedef typename RT<R>::R2 R2;
    typedef typename RT<R>::R4 R4;
    int G = 0, N = 0, E = 0, threads = 512, npt = 2;
    cudaStream_t s = nullptr;
    DevMem mem;
    BatchArrays<R> A{};
    BatchGraph *graphs = nullptr;
    int *queue = nullptr, *next = nullptr, *status = nullptr;
    std::vector<int> node0, nsize;
    int blocks = 0;
    std::map<int, cudaGraphExec_t> execs; // iteration count -> captured launch

    ~Batch() override
    {
        if (s) cudaStreamSynchronize(s);
        drop_graphs();
        mem.release();
        if (s) cudaStreamDestroy(s);
    }

    cudaStream_t stream() override { return s; }
    double bytes() const override { return mem.bytes; }
    int count() const override { return G; }

    int open(const fa2_full_params *ps, int count, const double *const *pos, int exact_below,
             int nthreads, int nodes_per_thread)
    {
        G = count;
        threads = nthreads;
        npt = nodes_per_thread;
        node0.resize(G);
        nsize.resize(G);
        bool any_adjust = false, any_fixed = false;
        std::vector<uint8_t> gfixed(G, 0); // graph g has a fixed node
        long long nn = 0, ee = 0;
        for (int g = 0; g < G; g++) {
            const fa2_full_params &p = ps[g];
            node0[g] = (int) nn;
            nsize[g] = p.n;
            nn += p.n;
            ee += p.inc_off[p.n];
            any_adjust |= p.adjust != 0;
            for (int i = 0; i < p.n && p.fixed && !gfixed[g]; i++) gfixed[g] = p.fixed[i] != 0;
            any_fixed |= gfixed[g] != 0;
        }
        if (nn >= (1LL << 31) / 2 || ee >= (1LL << 31)) {
            set_message("the batch is too large (at most 2^30 nodes and 2^31 incidences)");
            return 1;
        }
        N = (int) nn;
        E = (int) ee;
        FA2_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking),
                "could not create a CUDA stream", 1);
        const size_t n1 = (size_t) N;
        A.pos = mem.get<R2>(n1);
        A.f = mem.get<R2>(n1);
        A.fold = mem.get<R2>(n1);
        A.mass = mem.get<R>(n1);
        A.size = any_adjust ? mem.get<R>(n1) : nullptr;
        A.sw = mem.get<R>(n1);
        A.tr = sizeof(R) == 8 ? mem.get<R>(n1) : nullptr;
        A.fixed = any_fixed ? mem.get<uint8_t>(n1) : nullptr;
        A.off = mem.get<int>(n1 + 1);
        A.inc = mem.get<Inc<R>>((size_t) E);
        A.key = mem.get<uint32_t>(n1);
        A.idx = mem.get<uint32_t>(n1);
        A.key_b = mem.get<uint32_t>(n1);
        A.idx_b = mem.get<uint32_t>(n1);
        A.psort = mem.get<R4>(n1);
        A.child = mem.get<int2>(n1);
        A.range = mem.get<int2>(n1);
        A.parent = mem.get<int>(2 * n1);
        A.rope = mem.get<int>(n1);
        A.visits = mem.get<int>(n1);
        A.agg = mem.get<Agg<R>>(n1);
        A.rec_c = mem.get<R4>(n1);
        A.rec_t = mem.get<int2>(n1);
        graphs = mem.get<BatchGraph>((size_t) G);
        queue = mem.get<int>((size_t) G);
        next = mem.get<int>(1);
        status = mem.get<int>(ST_COUNT);
        if (mem.failed) {
            set_cuda_error("could not allocate memory on the device", mem.err);
            return 1;
        }
        // the graphs, concatenated on the host in the device precision
        std::vector<R2> hp(n1);
        std::vector<R> hm(n1), hs(any_adjust ? n1 : 0);
        std::vector<uint8_t> hf(any_fixed ? n1 : 0);
        std::vector<int> hoff(n1 + 1);
        std::vector<Inc<R>> hinc((size_t) std::max(E, 1));
        std::vector<BatchGraph> hg(G);
        int e0 = 0;
        for (int g = 0; g < G; g++) {
            const fa2_full_params &p = ps[g];
            const int n = p.n, b = node0[g];
            for (int i = 0; i < n; i++) {
                hp[b + i] = mk2h(pos[g][i], pos[g][n + i]);
                hm[b + i] = (R) p.mass[i];
                if (any_adjust) hs[b + i] = p.adjust ? (R) p.size[i] : R(0);
                if (any_fixed) hf[b + i] = gfixed[g] && p.fixed[i] != 0;
                hoff[b + i] = e0 + p.inc_off[i];
            }
            for (int e = 0; e < p.inc_off[n]; e++) {
                hinc[e0 + e].j = p.inc_node[e];
                hinc[e0 + e].coef = (R) p.inc_coef[e];
            }
            e0 += p.inc_off[n];
            BatchGraph &q = hg[g];
            memset(&q, 0, sizeof(q));
            q.n = n;
            q.node0 = b;
            q.exact = n < exact_below ? 1 : 0;
            int fl = 0;
            if (p.strong) fl |= BF_STRONG;
            if (p.linlog) fl |= BF_LINLOG;
            if (p.adjust) fl |= BF_ADJUST;
            if (gfixed[g]) fl |= BF_FIXED;
            for (int i = 0; i < n; i++)
                if ((float) p.mass[i] >= HUB_MASS) {
                    fl |= BF_HUBS;
                    break;
                }
            q.flags = fl;
            q.scaling = p.scaling;
            q.gravity = p.gravity;
            q.theta2d = p.theta * p.theta;
            q.jitter = p.jitter_tolerance;
            q.speed = 1.0;
            q.efficiency = 1.0;
        }
        hoff[n1] = e0;
        // largest work first: a block that takes a graph lays it out to the end
        std::vector<int> hq(G);
        std::iota(hq.begin(), hq.end(), 0);
        std::stable_sort(hq.begin(), hq.end(), [&](int a, int b) {
            const double ca = hg[a].exact ? (double) hg[a].n * hg[a].n : 300.0 * hg[a].n;
            const double cb = hg[b].exact ? (double) hg[b].n * hg[b].n : 300.0 * hg[b].n;
            return ca > cb;
        });
        int rc = 0;
        auto up = [&](void *dst, const void *src, size_t bytes) {
            if (!rc && bytes)
                rc = cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, s) != cudaSuccess;
        };
        up(A.pos, hp.data(), n1 * sizeof(R2));
        up(A.mass, hm.data(), n1 * sizeof(R));
        if (any_adjust) up(A.size, hs.data(), n1 * sizeof(R));
        if (any_fixed) up(A.fixed, hf.data(), n1);
        up(A.off, hoff.data(), (n1 + 1) * sizeof(int));
        up(A.inc, hinc.data(), (size_t) E * sizeof(Inc<R>));
        up(graphs, hg.data(), (size_t) G * sizeof(BatchGraph));
        up(queue, hq.data(), (size_t) G * sizeof(int));
        if (!rc) rc = cudaMemsetAsync(A.fold, 0, n1 * sizeof(R2), s) != cudaSuccess;
        if (!rc) rc = cudaMemsetAsync(status, 0, ST_COUNT * sizeof(int), s) != cudaSuccess;
        if (!rc) rc = cudaStreamSynchronize(s) != cudaSuccess;
        if (rc) {
            set_cuda_error("could not send the batch to the device", cudaGetLastError());
            return 1;
        }
        int sms = 0, per_sm = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (threads == 256)
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<R, 256>, 256, 0);
        else
            cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<R, 512>, 512, 0);
        blocks = std::max(1, std::min(G, sms * std::max(per_sm, 1)));
        return 0;
    }

    static R2 mk2h(double x, double y)
    {
        R2 v;
        v.x = (R) x;
        v.y = (R) y;
        return v;
    }

    void launch(int iterations)
    {
        cudaMemsetAsync(next, 0, sizeof(int), s);
        if (threads == 256)
            k_batch<R, 256><<<blocks, 256, 0, s>>>(G, graphs, queue, next, iterations, A, npt,
                                                   status);
        else
            k_batch<R, 512><<<blocks, 512, 0, s>>>(G, graphs, queue, next, iterations, A, npt,
                                                   status);
    }

    // The work-counter reset and the persistent launch, captured once per
    // iteration count (a few counts kept) and replayed.
    int iterate(int iterations) override
    {
        cudaSetDevice(device);
        auto it = execs.find(iterations);
        if (it == execs.end()) {
            if (execs.size() >= 8) drop_graphs();
            cudaGraph_t g = nullptr;
            cudaGraphExec_t x = nullptr;
            FA2_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                    "could not capture the batched launch", 1);
            launch(iterations);
            cudaError_t e = cudaStreamEndCapture(s, &g);
            if (e == cudaSuccess) e = cudaGraphInstantiate(&x, g, 0);
            if (g) cudaGraphDestroy(g);
            if (e != cudaSuccess) {
                set_cuda_error("could not capture the batched launch", e);
                return 1;
            }
            it = execs.emplace(iterations, x).first;
        }
        FA2_TRY(cudaGraphLaunch(it->second, s), "the computation on the GPU failed", 1);
        return 0;
    }

    void drop_graphs()
    {
        for (auto &kv : execs) cudaGraphExecDestroy(kv.second);
        execs.clear();
    }

    // Cycles of each phase, summed over the blocks, over `iterations`
    // iterations of every graph (an uncaptured, instrumented launch).
    int phase_cycles(int iterations, double out[8]) override
    {
        cudaSetDevice(device);
        DevMem tmp;
        unsigned long long *prof = tmp.get<unsigned long long>((size_t) blocks * 8);
        if (tmp.failed) {
            set_cuda_error("could not allocate memory on the device", tmp.err);
            return 1;
        }
        int rc = cudaMemsetAsync(prof, 0, (size_t) blocks * 8 * sizeof(unsigned long long), s) !=
                 cudaSuccess;
        BatchArrays<R> P = A;
        P.prof = prof;
        if (!rc) rc = cudaMemsetAsync(next, 0, sizeof(int), s) != cudaSuccess;
        if (!rc) {
            if (threads == 256)
                k_batch<R, 256><<<blocks, 256, 0, s>>>(G, graphs, queue, next, iterations, P,
                                                       npt, status);
            else
                k_batch<R, 512><<<blocks, 512, 0, s>>>(G, graphs, queue, next, iterations, P,
                                                       npt, status);
        }
        std::vector<unsigned long long> h((size_t) blocks * 8);
        if (!rc)
            rc = cudaMemcpyAsync(h.data(), prof, h.size() * sizeof(unsigned long long),
                                 cudaMemcpyDeviceToHost, s) != cudaSuccess;
        if (!rc) rc = cudaStreamSynchronize(s) != cudaSuccess;
        tmp.release();
        if (rc) {
            set_message("the computation on the GPU failed");
            return 1;
        }
        for (int k = 0; k < 8; k++) out[k] = 0.0;
        for (size_t b = 0; b < (size_t) blocks; b++)
            for (int k = 0; k < 8; k++) out[k] += (double) h[b * 8 + k];
        return 0;
    }

    int sync() override
    {
        cudaSetDevice(device);
        FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
        int h = 0;
        FA2_TRY(cudaMemcpy(&h, status + ST_ERROR, sizeof(int), cudaMemcpyDeviceToHost),
                "the computation on the GPU failed", 1);
        if (h & ERR_NAN) {
            set_message("the computation on the GPU produced invalid numbers");
            return 1;
        }
        if (h) {
            set_message("the computation on the GPU failed (an index left its bounds)");
            return 1;
        }
        return 0;
    }

    int positions(int g, double *out) override
    {
        if (g < 0 || g >= G) {
            set_message("there is no graph %d in this batch", g + 1);
            return 1;
        }
        cudaSetDevice(device);
        const int n = nsize[g];
        std::vector<R2> h((size_t) n);
        FA2_TRY(cudaMemcpyAsync(h.data(), A.pos + node0[g], (size_t) n * sizeof(R2),
                                cudaMemcpyDeviceToHost, s),
                "could not fetch the layout from the device", 1);
        FA2_TRY(cudaStreamSynchronize(s), "could not fetch the layout from the device", 1);
        for (int i = 0; i < n; i++) {
            out[i] = (double) h[i].x;
            out[n + i] = (double) h[i].y;
        }
        return 0;
    }

    // Graph g's forces of the last iteration (at the positions before its
    // displacement): the move keeps them in f.
    int forces(int g, double *out) override
    {
        if (g < 0 || g >= G) {
            set_message("there is no graph %d in this batch", g + 1);
            return 1;
        }
        cudaSetDevice(device);
        const int n = nsize[g];
        std::vector<R2> h((size_t) n);
        FA2_TRY(cudaMemcpyAsync(h.data(), A.f + node0[g], (size_t) n * sizeof(R2),
                                cudaMemcpyDeviceToHost, s),
                "could not fetch the forces from the device", 1);
        FA2_TRY(cudaStreamSynchronize(s), "could not fetch the forces from the device", 1);
        for (int i = 0; i < n; i++) {
            out[i] = (double) h[i].x;
            out[n + i] = (double) h[i].y;
        }
        return 0;
    }
    int speed(int g, double state[4]) override
    {
        if (g < 0 || g >= G) {
            set_message("there is no graph %d in this batch", g + 1);
            return 1;
        }
        BatchGraph h;
        FA2_TRY(cudaMemcpy(&h, graphs + g, sizeof(h), cudaMemcpyDeviceToHost), "cudaMemcpy", 1);
        state[0] = h.speed;
        state[1] = h.efficiency;
        state[2] = h.total_swinging;
        state[3] = h.total_traction;
        return 0;
    }

};

template <class R>
BatchBase *make_batch(const fa2_full_params *ps, int count, const double *const *pos,
                      int exact_below, int threads, int npt)
{
    const int dev = ps[0].device;
    FA2_TRY(cudaSetDevice(dev), "could not use the CUDA device", nullptr);
    Batch<R> *B = new Batch<R>();
    B->device = dev;
    if (B->open(ps, count, pos, exact_below, threads, npt)) {
        delete B;
        return nullptr;
    }
    return B;
}

// ---- autotuner -------------------------------------------------------------------
// The exact-vs-Barnes-Hut crossover, the block size and the exact sum's tile
// shape, measured on the device: Erdos-Renyi graphs (mean degree 8), two per
// SM, laid out for 2 iterations (after 2) in each mode, at 64, 128, .. 16384
// nodes until the tree is faster, then at quarter-octave sizes below that
// one; the crossover is the smallest size measured at which the tree is
// faster. Block sizes 256 and 512 are compared on 2048-node graphs; then 1
// or 2 nodes per thread of the exact sum on graphs of 3/4 of the crossover
// (at least one block of nodes more).

struct TuneGraphs {
    std::vector<std::vector<int>> off, node;
    std::vector<std::vector<double>> coef, mass, size, pos;
    std::vector<fa2_full_params> ps;
    std::vector<const double *> pp;
};

static uint64_t splitmix(uint64_t &x)
{
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static void tune_graphs(TuneGraphs &t, int n, int copies, int device, int use_double)
{
    t.off.resize(copies);
    t.node.resize(copies);
    t.coef.resize(copies);
    t.mass.resize(copies);
    t.size.resize(copies);
    t.pos.resize(copies);
    t.ps.resize(copies);
    t.pp.resize(copies);
    uint64_t seed = 12345 + (uint64_t) n;
    for (int c = 0; c < copies; c++) {
        const int m = 4 * n;
        std::vector<int> a(m), b(m), deg(n, 0);
        for (int e = 0; e < m; e++) {
            a[e] = (int) (splitmix(seed) % (uint64_t) n);
            b[e] = (int) (splitmix(seed) % (uint64_t) n);
            if (a[e] == b[e]) b[e] = (b[e] + 1) % n;
            deg[a[e]]++;
            deg[b[e]]++;
        }
        auto &off = t.off[c];
        off.assign(n + 1, 0);
        for (int i = 0; i < n; i++) off[i + 1] = off[i] + deg[i];
        std::vector<int> at(off.begin(), off.end() - 1);
        t.node[c].resize(2 * m);
        t.coef[c].assign(2 * m, 1.0);
        for (int e = 0; e < m; e++) {
            t.node[c][at[a[e]]++] = b[e];
            t.node[c][at[b[e]]++] = a[e];
        }
        t.mass[c].resize(n);
        t.size[c].assign(n, 1.0);
        for (int i = 0; i < n; i++) t.mass[c][i] = 1.0 + deg[i];
        t.pos[c].resize(2 * n);
        const double r = 10.0 * std::sqrt((double) n);
        for (int i = 0; i < 2 * n; i++)
            t.pos[c][i] = r * (2.0 * (double) (splitmix(seed) >> 11) / 9007199254740992.0 - 1.0);
        fa2_full_params &p = t.ps[c];
        memset(&p, 0, sizeof(p));
        p.n = n;
        p.inc_off = off.data();
        p.inc_node = t.node[c].data();
        p.inc_coef = t.coef[c].data();
        p.mass = t.mass[c].data();
        p.size = t.size[c].data();
        p.scaling = 2.0;
        p.gravity = 1.0;
        p.theta = 1.2;
        p.jitter_tolerance = 1.0;
        p.device = device;
        p.use_double = use_double;
        t.pp[c] = t.pos[c].data();
    }
}

// Milliseconds per graph-iteration of a batch of these graphs (-1 on error).
template <class R>
static double time_batch(TuneGraphs &t, int exact_below, int threads, int npt = 2)
{
    BatchBase *B =
        make_batch<R>(t.ps.data(), (int) t.ps.size(), t.pp.data(), exact_below, threads, npt);
    if (!B) return -1.0;
    double ms = -1.0;
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    if (!B->iterate(2)) { // warm-up; also captures the timed launch
        cudaEventRecord(e0, B->stream());
        if (!B->iterate(2)) {
            cudaEventRecord(e1, B->stream());
            if (!B->sync()) {
                float f = 0.f;
                cudaEventElapsedTime(&f, e0, e1);
                ms = f / (2.0 * (double) t.ps.size());
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    delete B;
    return ms;
}

template <class R> int tune_batch(int device, int *exact_below, int *threads, int *npt)
{
    int sms = 0;
    FA2_TRY(cudaSetDevice(device), "could not use the CUDA device", 1);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int copies = 2 * std::max(sms, 1);
    // 1: tree faster, 0: exact faster, -1: error
    auto tree_wins = [&](int n) {
        TuneGraphs t;
        tune_graphs(t, n, copies, device, sizeof(R) == 8);
        const double te = time_batch<R>(t, 1 << 30, 512);
        const double tb = time_batch<R>(t, 0, 512);
        if (te < 0 || tb < 0) return -1;
        return tb < te ? 1 : 0;
    };
    // the first power of two at which the tree wins, then quarter-octave
    // steps below it
    int hi = 0;
    for (int n = 64; n <= 16384; n *= 2) {
        const int w = tree_wins(n);
        if (w < 0) return 1;
        if (w) {
            hi = n;
            break;
        }
    }
    int cross = hi ? hi : 32768;
    if (hi > 64) {
        for (int q = 1; q < 4; q++) {
            const int n = (int) std::lround((hi / 2) * std::pow(2.0, q / 4.0));
            const int w = tree_wins(n);
            if (w < 0) return 1;
            if (w) {
                cross = n;
                break;
            }
        }
    }
    TuneGraphs t;
    tune_graphs(t, 2048, copies, device, sizeof(R) == 8);
    const double t256 = time_batch<R>(t, 0, 256), t512 = time_batch<R>(t, 0, 512);
    if (t256 < 0 || t512 < 0) return 1;
    const int th = t256 < t512 ? 256 : 512;
    TuneGraphs u;
    tune_graphs(u, std::min(std::max(cross * 3 / 4, th + 1), 4096), copies, device,
                sizeof(R) == 8);
    const double t1 = time_batch<R>(u, 1 << 30, th, 1), t2 = time_batch<R>(u, 1 << 30, th, 2);
    if (t1 < 0 || t2 < 0) return 1;
    *exact_below = cross;
    *threads = th;
    *npt = t1 < t2 ? 1 : 2;
    return 0;
}

} // namespace fa2cu

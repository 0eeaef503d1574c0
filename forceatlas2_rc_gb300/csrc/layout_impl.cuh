// layout_impl.cuh -- the device sessions, templated on the real type.
// Included by inst_f32.cu and inst_f64.cu only, so that every kernel they
// launch is compiled with the flags of its precision.
//
// HBM layout of a Layout<R> (n nodes, E incidences; float sizes):
//   pos, f, fold        R2[n]   positions, forces, previous forces
//   mass, size, sw      R[n]    masses, radii (adjust), swinging
//   fixed               u8[n]   (when some node is fixed)
//   inc_off, inc        int[n+1], {int j; R coef}[E]  symmetric CSR
//   key, order (+ ping-pong)  u32[n] x 4, look-back words u32[4 * 256 * n / 2048]
//   psort               R4[n]   (x, y, m, r) in Morton order
//   child, range        int2[n-1], parent int[2n-1], rope int[n],
//   visits              int[n-1], agg Agg<R>[n-1] (double / float-float sums),
//                       rec_c R4[n-1], rec_t int2[n-1] (traversal records)
//   bbox, quant         the bounding box and Morton quantisation, computed by
//                       the displacement of the previous iteration
//   packed, exact_part  R4[n], R2[rows n]  (exact repulsion only)
//   st, status          FP64 speed state, status words
#pragma once

#include <stdio.h>
#include <string.h>
#include <time.h>
#include <vector>

#include "devmem.cuh"
#include "kernels.cuh"
#include "prep.cuh"
#include "session.h"
#include "sort_tree.cuh"

namespace fa2cu {

inline double now_s()
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double) ts.tv_sec + 1e-9 * (double) ts.tv_nsec;
}

// The all-pairs repulsion of n packed records into f: k_exact over `rows`
// source ranges (exact_rows), then their fixed-order sum when rows > 1
// (partial holds rows * n entries).
template <class R, int IPT>
void launch_exact(cudaStream_t s, int n, bool adjust, R scaling, const typename RT<R>::R4 *packed,
                  typename RT<R>::R2 *f, typename RT<R>::R2 *partial, int rows, int *status)
{
    constexpr int TILE = exact_tile<R>();
    const int seg = rows > 1 ? ceil_div(ceil_div(n, rows), TILE) * TILE : ceil_div(n, TILE) * TILE;
    rows = ceil_div(n, seg);
    const dim3 grid(ceil_div(n, FA2_EXACT_THREADS * IPT), rows);
    const size_t smem = exact_smem_bytes<R>();
    typename RT<R>::R2 *part = rows > 1 ? partial : nullptr;
    if (adjust)
        k_exact<R, true, IPT><<<grid, FA2_EXACT_THREADS, smem, s>>>(n, scaling, packed, f, part,
                                                                    seg, status);
    else
        k_exact<R, false, IPT><<<grid, FA2_EXACT_THREADS, smem, s>>>(n, scaling, packed, f, part,
                                                                     seg, status);
    if (rows > 1) k_exact_sum<R><<<ceil_div(n, 256), 256, 0, s>>>(n, rows, partial, f);
}

template <class R> struct Layout : LayoutBase {
    typedef typename RT<R>::R2 R2;
    typedef typename RT<R>::R4 R4;

    int n = 0, ninc = 0, repulsion = 0, adjust = 0, strong = 0, linlog = 0;
    int any_fixed = 0;
    // FP32: the walk with deferred node pairs (0.48-0.52 against 0.57-0.61
    // ms at 10^6 nodes); FP64: one walk per thread, in the reference's
    // order of the forces
    int walk = sizeof(R) == 4 ? WALK_DEFERRED : WALK_THREAD;
    int climb_mode = 1; // leaves per aggregate thread (negative: interleaved)
    bool block_sort = false; // few keys: the one-block sort

    // Leaves per thread of the tree's climb, from the ratio x of leaves to
    // the threads the device holds at once (1536 per SM in float, 40
    // registers). With block-local arrivals and the links of the next level
    // loaded early (gather + Karras + climb in ms for 1 / 2 / 4 / 8 leaves
    // per thread): BA 1e5 (x 0.43) 0.052 / 0.054 / 0.057 / 0.070; SBM 3e5
    // (x 1.3) 0.071 / 0.066 / 0.066 / 0.078; 1e6 (x 4.3) 0.141 / 0.126 /
    // 0.148 / 0.144; 3e6 0.346 / 0.276 / 0.287 / 0.405. Earlier build (2048
    // threads per SM, device-scope arrivals only; climb alone, 1 / 2 / 4 / 8
    // leaves per thread): 2e5 leaves (x 0.64) 0.069 / 0.074 / 0.084 / 0.123;
    // 4e5 (x 1.3) 0.101 / 0.091 / 0.100 / 0.142; 6e5 (x 1.9) 0.128 / 0.107 /
    // 0.117 / 0.155; 1e6 (x 3.2) 0.186 / 0.157 / 0.159 / 0.199; 2e6 (x 6.4)
    // 0.326 / 0.263 / 0.289 / 0.387; 3e6 (x 9.6) 0.459 / 0.355 / 0.410 /
    // 0.629. FP64 (fewer threads per SM): 4 leaves per thread was fastest or
    // tied at 1e5 and 1e6 leaves (1e6: 0.554 / 0.382 / 0.334).
    static int pick_climb(int n, int device)
    {
        if (sizeof(R) == 8) return n >= 50000 ? 4 : 1;
        int sms = 0, blocks = 0;
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, k_aggregate_multi<R, 2, true>,
                                                          256, 0) !=
                cudaSuccess ||
            blocks < 1 || sms < 1) {
            cudaGetLastError();
            return 1;
        }
        const double x = (double) n / ((double) sms * blocks * 256.0);
        return x < 1.0 ? 1 : 2;
    }
    R scaling = 0, gravity = 0, theta2 = 0;
    R wscale = 0; // FP32 records: size^2 (1 + DECIDE_BAND) / theta^2 (region_far)
    double theta2d = 0.0;
    cudaStream_t s = nullptr;
    DevMem mem;
    R2 *pos = nullptr, *f = nullptr, *fold = nullptr;
    R *mass = nullptr, *size = nullptr, *sw = nullptr, *trac = nullptr;
    uint8_t *fixed = nullptr;
    int *inc_off = nullptr;
    Inc<R> *inc = nullptr;
    // FP32: the nodes of HEAVY_DEGREE incidences or more (heavy_cap of room,
    // then their count), summed by a warp each
    int *heavy = nullptr;
    int heavy_cap = 0, nheavy = 0;
    int launches = 0; // kernels of one captured iteration
    R *bbox = nullptr, *bbox_partial = nullptr;
    double *quant = nullptr; // min x, min y, Morton scale, -, 4 floats (k_bbox)
    int nbbox = 1;
    uint32_t *key = nullptr, *order = nullptr;
    SortScratch ss{};
    R4 *psort = nullptr, *packed = nullptr;
    R2 *exact_part = nullptr; // exact_rows rows of partial sums (rows > 1)
    int exact_nrows = 1;
    int2 *child = nullptr, *range = nullptr;
    int *parent = nullptr, *rope = nullptr, *visits = nullptr;
    Agg<R> *agg = nullptr;
    R4 *rec_c = nullptr; // traversal records (common.cuh)
    int2 *rec_t = nullptr;
    double2 *swing_partial = nullptr;
    SpeedState *st = nullptr;
    int *status = nullptr;
    double *xy = nullptr; // 2n doubles of staging
    unsigned long long *counts = nullptr;
    cudaGraphExec_t g1 = nullptr, g8 = nullptr;
    cudaEvent_t ev[8] = {};
    // FP32 Barnes-Hut: the attraction on a second stream beside the tree
    // build and the walk, into its own buffer fatt, on attract_grid blocks
    // per SM (beside())
    int overlap = sizeof(R) == 4 ? 1 : 0, attract_grid = 1;
    // grid of the join: 4 blocks per SM, grid-stride (0.709-0.712 -> 0.703
    // ms an iteration at 10^6 SBM nodes against one block per 256 nodes,
    // whose last block added 3907 partials)
    int join_blocks = 152 * 4;
    // the iteration's kernels on the main stream launched as programmatic
    // dependents (launch_k; option "pdl"), below 500,000 nodes: ms an
    // iteration without / with, SBM 10^4 0.1435 / 0.1411, BA 10^5 0.2018 /
    // 0.1988, SBM 10^6 0.6799 / 0.6855 (positions identical)
    bool pdl = false;
    cudaStream_t s2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    R2 *fatt = nullptr;

    ~Layout() override
    {
        if (s) cudaStreamSynchronize(s);
        if (g1) cudaGraphExecDestroy(g1);
        if (g8) cudaGraphExecDestroy(g8);
        for (auto &e : ev)
            if (e) cudaEventDestroy(e);
        mem.release();
        if (ev_fork) cudaEventDestroy(ev_fork);
        if (ev_join) cudaEventDestroy(ev_join);
        if (s2) cudaStreamDestroy(s2);
        if (s) cudaStreamDestroy(s);
    }

    double bytes() const override { return mem.bytes; }
    cudaStream_t stream() override { return s; }

    int alloc(bool want_tree)
    {
        const size_t nn = (size_t) n;
        pos = mem.get<R2>(nn);
        f = mem.get<R2>(nn);
        fold = mem.get<R2>(nn);
        mass = mem.get<R>(nn);
        size = adjust ? mem.get<R>(nn) : nullptr;
        sw = mem.get<R>(nn);
        trac = serial_totals<R>(n) ? mem.get<R>(nn) : nullptr;
        fixed = any_fixed ? mem.get<uint8_t>(nn) : nullptr;
        inc_off = mem.get<int>(nn + 1);
        inc = mem.get<Inc<R>>((size_t) ninc);
        if (sizeof(R) == 4) {
            heavy_cap = ninc / HEAVY_DEGREE;
            heavy = mem.get<int>((size_t) heavy_cap + 1);
        }
        swing_partial = mem.get<double2>((size_t) ceil_div(n, 256)); // one per block
        st = mem.get<SpeedState>(1);
        status = mem.get<int>(ST_COUNT);
        xy = mem.get<double>(2 * nn);
        counts = mem.get<unsigned long long>(2);
        if (want_tree) {
            nbbox = std::min(ceil_div(n, 256), 152 * 4);
            bbox = mem.get<R>(4);
            quant = mem.get<double>(6);
            bbox_partial = mem.get<R>(4 * (size_t) nbbox);
            key = mem.get<uint32_t>(nn);
            order = mem.get<uint32_t>(nn);
            ss.key_b = mem.get<uint32_t>(nn);
            ss.val_b = mem.get<uint32_t>(nn);
            ss.counts = mem.get<uint32_t>(sort_scratch_counts(n));
            ss.err = status + ST_ERROR;
            ss.digit_total = mem.get<uint32_t>(SORT_AUX);
            psort = mem.get<R4>(nn);
            child = mem.get<int2>(nn - 1);
            range = mem.get<int2>(nn - 1);
            parent = mem.get<int>(2 * nn - 1);
            rope = mem.get<int>(nn);
            visits = mem.get<int>(nn - 1);
            agg = mem.get<Agg<R>>(nn - 1);
            rec_c = mem.get<R4>(nn - 1);
            rec_t = mem.get<int2>(nn - 1);
            if (sizeof(R) == 4) fatt = mem.get<R2>(nn);
        } else {
            packed = mem.get<R4>(nn);
            if (exact_nrows > 1) exact_part = mem.get<R2>((size_t) exact_nrows * nn);
        }
        if (mem.failed) {
            set_cuda_error("could not allocate memory on the device", mem.err);
            return 1;
        }
        return 0;
    }

    // The graph from its edge list, prepared on the device (prep.cu): the
    // masses, the incidence lists and their coefficients in double, then
    // converted to the layout's precision.
    int prepare_edges(const fa2_full_params *p, const EdgeList &E)
    {
        DevMem tmp;
        tmp.pool = mem.pool;
        tmp.s = s;
        const size_t m1 = (size_t) std::max(E.m, 1);
        int *from = tmp.get<int>(m1), *to = tmp.get<int>(m1);
        double *w = tmp.get<double>(m1);
        double *dmass = tmp.get<double>((size_t) n);
        int *dnode = tmp.get<int>(2 * m1);
        double *dcoef = tmp.get<double>(std::max(2 * m1, (size_t) n));
        PrepScratch ws;
        prep_scratch(tmp, n, E.m, ws);
        if (tmp.failed) {
            tmp.release();
            set_cuda_error("could not allocate memory on the device", tmp.err);
            return 1;
        }
        int rc = 0;
        auto up = [&](void *dst, const void *src, size_t b) {
            if (!rc && b) rc = cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, s) != cudaSuccess;
        };
        up(from, E.from, (size_t) E.m * sizeof(int));
        up(to, E.to, (size_t) E.m * sizeof(int));
        up(w, E.w, (size_t) E.m * sizeof(double));
        if (rc) {
            tmp.release();
            set_cuda_error("could not send the graph to the device", cudaGetLastError());
            return 1;
        }
        const long long got =
            prep_graph(s, n, E.m, from, to, w, E.outbound, dmass, inc_off, dnode, dcoef, ws);
        if (got < 0) {
            cudaStreamSynchronize(s);
            tmp.release();
            return 1;
        }
        ninc = (int) got;
        k_real_in<R><<<ceil_div(n, 256), 256, 0, s>>>(n, dmass, mass);
        if (ninc > 0) k_inc_in<R><<<ceil_div(ninc, 256), 256, 0, s>>>(ninc, dnode, dcoef, inc);
        if (adjust) {
            up(dcoef, p->size, (size_t) n * sizeof(double));
            if (!rc) k_real_in<R><<<ceil_div(n, 256), 256, 0, s>>>(n, dcoef, size);
        }
        if (any_fixed) {
            std::vector<uint8_t> f8((size_t) n);
            for (int i = 0; i < n; i++) f8[i] = p->fixed[i] != 0;
            up(fixed, f8.data(), (size_t) n);
        }
        if (!rc) rc = cudaStreamSynchronize(s) != cudaSuccess;
        tmp.release();
        if (rc) {
            set_cuda_error("could not send the graph to the device", cudaGetLastError());
            return 1;
        }
        return 0;
    }

    int open(const fa2_full_params *p, const double *xy0, int rep,
             const LayoutOpts *opts = nullptr, const EdgeList *edges = nullptr)
    {
        n = p->n;
        // from an edge list: at most two incidences per edge until the
        // preparation on the device has counted them
        ninc = edges ? 2 * edges->m : p->inc_off[n];
        repulsion = rep;
        adjust = p->adjust ? 1 : 0;
        strong = p->strong ? 1 : 0;
        linlog = p->linlog ? 1 : 0;
        any_fixed = 0;
        if (p->fixed)
            for (int i = 0; i < n && !any_fixed; i++) any_fixed = p->fixed[i] != 0;
        scaling = (R) p->scaling;
        gravity = (R) p->gravity;
        theta2d = p->theta * p->theta;
        theta2 = (R) theta2d;
        wscale = (R) ((1.0 + (double) DECIDE_BAND) / theta2d);
        if (opts && opts->has_priority)
            FA2_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, opts->priority),
                    "could not create a CUDA stream", 1);
        else
            FA2_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking),
                    "could not create a CUDA stream", 1);
        for (auto &e : ev) FA2_TRY(cudaEventCreate(&e), "could not create a CUDA event", 1);
        if (sizeof(R) == 4 && rep == FA2CU_REPULSION_BH) {
            FA2_TRY(cudaStreamCreateWithFlags(&s2, cudaStreamNonBlocking),
                    "could not create a CUDA stream", 1);
            FA2_TRY(cudaEventCreateWithFlags(&ev_fork, cudaEventDisableTiming),
                    "could not create a CUDA event", 1);
            FA2_TRY(cudaEventCreateWithFlags(&ev_join, cudaEventDisableTiming),
                    "could not create a CUDA event", 1);
        }

        mem.pool = opts ? opts->pool : nullptr;
        mem.s = s;
        if (rep == FA2CU_REPULSION_BH && sort_setup()) return 1;
        if (rep == FA2CU_REPULSION_BH) {
            climb_mode = pick_climb(n, device);
            // sort tiles: fewer than ~75 tiles of 8192 keys leave most SMs
            // idle; measured on a GB300 (sort of one iteration, ms, tiles of
            // 256 / 512 / 1024 threads): 1e5 keys 0.050 / 0.051 / 0.060;
            // 3e5 0.054 / 0.054 / 0.066; 1e6 0.092 / 0.077 / 0.070; 3e6
            // 0.178 / 0.164 / 0.163
            ss.tile_threads = n < 600000 ? 512 : 1024;
            pdl = n < 500000;
            ss.pdl = pdl;
            block_sort = n <= SORT_BLOCK_MAX;
        }
        if (rep == FA2CU_REPULSION_EXACT) {
            int sms = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
            exact_nrows = exact_rows<R>(n, std::max(sms, 1), EXACT_IPT);
        }
        if (alloc(rep == FA2CU_REPULSION_BH)) return 1;

        // the graph, once (reference src/gpu_full.c:241-287), or prepared on
        // the device from its edge list
        if (edges) {
            if (prepare_edges(p, *edges)) return 1;
        } else {
            DevMem tmp;
            tmp.pool = mem.pool;
            tmp.s = s;
            double *dd = tmp.get<double>(std::max<size_t>((size_t) n, (size_t) ninc));
            int *di = tmp.get<int>((size_t) ninc);
            if (tmp.failed) {
                tmp.release();
                set_cuda_error("could not allocate memory on the device", tmp.err);
                return 1;
            }
            int rc = 0;
            auto up = [&](void *dst, const void *src, size_t b) {
                if (!rc && b) rc = cudaMemcpyAsync(dst, src, b, cudaMemcpyHostToDevice, s) != cudaSuccess;
            };
            up(dd, p->mass, (size_t) n * sizeof(double));
            if (!rc) k_real_in<R><<<ceil_div(n, 256), 256, 0, s>>>(n, dd, mass);
            if (adjust) {
                up(dd, p->size, (size_t) n * sizeof(double));
                if (!rc) k_real_in<R><<<ceil_div(n, 256), 256, 0, s>>>(n, dd, size);
            }
            up(inc_off, p->inc_off, ((size_t) n + 1) * sizeof(int));
            if (ninc > 0) {
                up(dd, p->inc_coef, (size_t) ninc * sizeof(double));
                up(di, p->inc_node, (size_t) ninc * sizeof(int));
                if (!rc) k_inc_in<R><<<ceil_div(ninc, 256), 256, 0, s>>>(ninc, di, dd, inc);
            }
            if (any_fixed) {
                std::vector<uint8_t> f8((size_t) n);
                for (int i = 0; i < n; i++) f8[i] = p->fixed[i] != 0;
                up(fixed, f8.data(), (size_t) n);
                if (!rc) rc = cudaStreamSynchronize(s) != cudaSuccess;
            }
            if (!rc) rc = cudaStreamSynchronize(s) != cudaSuccess;
            tmp.release();
            if (rc) {
                set_cuda_error("could not send the graph to the device", cudaGetLastError());
                return 1;
            }
        }
        // the heavy nodes (FP32), listed once
        if (heavy) {
            FA2_TRY(cudaMemsetAsync(heavy + heavy_cap, 0, sizeof(int), s), "cudaMemset", 1);
            if (heavy_cap > 0)
                k_heavy_list<<<ceil_div(n, 256), 256, 0, s>>>(n, inc_off, heavy, heavy_cap);
            FA2_TRY(cudaMemcpyAsync(&nheavy, heavy + heavy_cap, sizeof(int),
                                    cudaMemcpyDeviceToHost, s),
                    "could not prepare the layout", 1);
            FA2_TRY(cudaStreamSynchronize(s), "could not prepare the layout", 1);
            nheavy = std::min(nheavy, heavy_cap);
        }
        // status words (error flags, arrival tickets) and the previous
        // forces start at zero; then the positions (and their bounding box,
        // whose reduction takes a ticket)
        FA2_TRY(cudaMemsetAsync(fold, 0, (size_t) n * sizeof(R2), s), "cudaMemset", 1);
        FA2_TRY(cudaMemsetAsync(status, 0, ST_COUNT * sizeof(int), s), "cudaMemset", 1);
        if (repulsion == FA2CU_REPULSION_BH) sort_prepare(s, ss);
        if (set_positions(xy0)) return 1;
        SpeedState h{};
        h.speed = 1.0;
        h.efficiency = 1.0;
        h.jitter_tolerance = p->jitter_tolerance;
        h.n = n;
        FA2_TRY(cudaMemcpyAsync(st, &h, sizeof(h), cudaMemcpyHostToDevice, s), "cudaMemcpy", 1);
        if (repulsion == FA2CU_REPULSION_EXACT) {
            const size_t smem = exact_smem_bytes<R>();
            FA2_TRY(cudaFuncSetAttribute(k_exact<R, false, EXACT_IPT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem),
                    "cudaFuncSetAttribute", 1);
            FA2_TRY(cudaFuncSetAttribute(k_exact<R, true, EXACT_IPT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem),
                    "cudaFuncSetAttribute", 1);
        }
        FA2_TRY(cudaStreamSynchronize(s), "could not prepare the layout", 1);
        if (capture(&g1, 1)) return 1;
        if (n <= (1 << 16) && capture(&g8, 8)) return 1;
        return 0;
    }

    static constexpr int EXACT_IPT = sizeof(R) == 4 ? FA2_EXACT_IPT_F32 : 1;

    // ---- the steps of one iteration ----
    // The bounding box and Morton quantisation of the current positions (the
    // displacement computes them for the positions it writes; this is for
    // positions set from outside).
    void launch_bbox()
    {
        k_bbox<R><<<nbbox, 256, 0, s>>>(n, pos, bbox_partial, bbox, quant,
                                        (unsigned *) (status + ST_TICKET_BBOX));
    }
    // Morton codes, with the sort's digit histograms in the same launch
    void launch_build()
    {
        const int nb = std::min(ceil_div(n, 256), 152 * 4);
        if (block_sort) { // the one-block sort counts its own digits
            k_morton<R><<<nb, 256, 0, s>>>(n, pos, quant, key, order, nullptr, nullptr, 0);
            return;
        }
        // the histograms, done counter and tickets start at zero: cleared at
        // open, then left at zero by the Morton kernel's last block for the
        // next sort (no memset in the iteration)
        launch_k(pdl, k_morton<R>, dim3(nb), dim3(256), 0, s, n, pos, quant, key, order,
                 ss.digit_total, ss.counts, sort_status_words(n, 4));
    }
    void launch_sort()
    {
        if (block_sort)
            sort_pairs_block(s, n, key, order, ss);
        else
            sort_pairs(s, n, key, order, ss, /*hist_ready=*/true);
    }
    void launch_tree()
    {
        launch_k(pdl, k_gather_karras<R>, dim3(ceil_div(n, 256)), dim3(256), 0, s, n, adjust,
                 order, pos, mass, size, psort, key, child, range, parent, rope, visits, status);
        // every climb kernel waits for its predecessor before reading the tree
        switch (climb_mode) {
        case 2:
            launch_k(pdl, k_aggregate_multi<R, 2, true>, dim3(ceil_div(n, 512)), dim3(256), 0, s,
                     n, psort, child, parent, range, rope, visits, agg, rec_c, rec_t, wscale,
                     status);
            break;
        case 4:
            launch_k(pdl, k_aggregate_multi<R, 4, true>, dim3(ceil_div(n, 1024)), dim3(256), 0,
                     s, n, psort, child, parent, range, rope, visits, agg, rec_c, rec_t, wscale,
                     status);
            break;
        case 8:
            launch_k(pdl, k_aggregate_multi<R, 8, true>, dim3(ceil_div(n, 2048)), dim3(256), 0,
                     s, n, psort, child, parent, range, rope, visits, agg, rec_c, rec_t, wscale,
                     status);
            break;
        case -2:
            launch_k(pdl, k_aggregate_multi<R, 2, false>, dim3(ceil_div(n, 512)), dim3(256), 0,
                     s, n, psort, child, parent, range, rope, visits, agg, rec_c, rec_t, wscale,
                     status);
            break;
        case -4:
            launch_k(pdl, k_aggregate_multi<R, 4, false>, dim3(ceil_div(n, 1024)), dim3(256), 0,
                     s, n, psort, child, parent, range, rope, visits, agg, rec_c, rec_t, wscale,
                     status);
            break;
        default:
            launch_k(pdl, k_aggregate<R>, dim3(ceil_div(n, 256)), dim3(256), 0, s, n, psort,
                     child, parent, range, rope, visits, agg, rec_c, rec_t, wscale, status);
        }
    }
    void launch_repulsion()
    {
        if (repulsion == FA2CU_REPULSION_BH) {
            if (walk == WALK_WARP) {
                if (adjust)
                    k_traverse_warp<R, true><<<ceil_div(n, 256), 256, 0, s>>>(
                        n, scaling, theta2, theta2d, psort, rec_c, rec_t, range, agg, rope, order, f,
                        status);
                else
                    k_traverse_warp<R, false><<<ceil_div(n, 256), 256, 0, s>>>(
                        n, scaling, theta2, theta2d, psort, rec_c, rec_t, range, agg, rope, order, f,
                        status);
            } else if (walk == WALK_THREAD) {
                if (adjust)
                    k_traverse<R, true, 6><<<ceil_div(n, 256), 256, 0, s>>>(
                        n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg, rope, order, f, status);
                else // float: 8 blocks per SM (0.597 against 0.619 ms at 6, 10^6 nodes)
                    k_traverse<R, false, sizeof(R) == 4 ? 8 : 6>
                        <<<ceil_div(n, 256), 256, 0, s>>>(n, scaling, theta2, theta2d, psort,
                                                          rec_c, rec_t, agg, rope, order, f,
                                                          status);
            } else if (walk == WALK_DEFERRED) {
                // graphs with hubs: their walks add up with compensation
                const int g = ceil_div(n, 256);
                // (every deferred walk waits for its predecessor first)
                if (adjust) {
                    if (nheavy > 0)
                        launch_k(pdl, k_traverse_deferred<R, true, 6, true>, dim3(g), dim3(256),
                                 0, s, n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg,
                                 rope, order, f, status);
                    else
                        launch_k(pdl, k_traverse_deferred<R, true, 6>, dim3(g), dim3(256), 0, s,
                                 n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg, rope,
                                 order, f, status);
                } else {
                    if (nheavy > 0)
                        launch_k(pdl, k_traverse_deferred<R, false, sizeof(R) == 4 ? 8 : 6, true>,
                                 dim3(g), dim3(256), 0, s, n, scaling, theta2, theta2d, psort,
                                 rec_c, rec_t, agg, rope, order, f, status);
                    else
                        launch_k(pdl, k_traverse_deferred<R, false, sizeof(R) == 4 ? 8 : 6>,
                                 dim3(g), dim3(256), 0, s, n, scaling, theta2, theta2d, psort,
                                 rec_c, rec_t, agg, rope, order, f, status);
                }
            } else if (walk == WALK_PAIR) {
                const int grid = ceil_div(ceil_div(n, 2), 256);
                if (adjust)
                    k_traverse_multi<R, true, 2><<<grid, 256, 0, s>>>(
                        n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg, rope, order, f, status);
                else
                    k_traverse_multi<R, false, 2><<<grid, 256, 0, s>>>(
                        n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg, rope, order, f, status);
            } else if (walk == WALK_QUAD) {
                const int grid = ceil_div(ceil_div(n, 4), 256);
                if (adjust)
                    k_traverse_multi<R, true, 4><<<grid, 256, 0, s>>>(
                        n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg, rope, order, f, status);
                else
                    k_traverse_multi<R, false, 4><<<grid, 256, 0, s>>>(
                        n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg, rope, order, f, status);
            } else {
                if (adjust)
                    k_traverse<R, true, 1><<<ceil_div(n, 256), 256, 0, s>>>(
                        n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg, rope, order, f, status);
                else
                    k_traverse<R, false, 1><<<ceil_div(n, 256), 256, 0, s>>>(
                        n, scaling, theta2, theta2d, psort, rec_c, rec_t, agg, rope, order, f, status);
            }
        } else {
            k_pack<R><<<ceil_div(n, 256), 256, 0, s>>>(n, adjust, pos, mass, size, packed);
            launch_exact<R, EXACT_IPT>(s, n, adjust, scaling, packed, f, exact_part, exact_nrows,
                                       status);
        }
    }
    // The heavy nodes' attraction (FP32), added to their repulsion.
    void launch_heavy()
    {
        if (nheavy > 0)
            k_attract_heavy<R><<<ceil_div(nheavy, 8), 256, 0, s>>>(nheavy, heavy, linlog, adjust,
                                                                  pos, size, inc_off, inc, f);
    }
    // Attraction and gravity only (the forces of fa2cu_layout_forces).
    void launch_attraction()
    {
        launch_heavy();
        k_attract<R><<<ceil_div(n, 256), 256, 0, s>>>(n, gravity, strong, linlog, adjust, pos,
                                                      mass, size, inc_off, inc, f);
    }
    // Attraction and gravity, swinging, traction, the totals and the speed
    // update (an iteration's second half before the displacement).
    void launch_attraction_swing()
    {
        // serial totals: the last block stages 2n reals
        const size_t smem = serial_totals<R>(n) ? 2 * (size_t) n * sizeof(R) : 0;
        launch_heavy();
        k_attract_swing<R><<<ceil_div(n, 256), 256, smem, s>>>(
            n, gravity, strong, linlog, adjust, pos, mass, size, inc_off, inc, f, fold, fixed, sw,
            trac, swing_partial, (unsigned *) (status + ST_TICKET_SWING), st, status);
    }
    // The displacement, with the next iteration's bounding box.
    void launch_move()
    {
        // with a tree, the bounding box's block count (its partials); else
        // one thread per node
        const int nb = bbox_partial ? nbbox : ceil_div(n, 256);
        launch_k(pdl, k_apply<R>, dim3(nb), dim3(256), 0, s, n, adjust, f, fold, sw, fixed, pos,
                 st, status, bbox_partial, bbox, quant, (unsigned *) (status + ST_TICKET_BBOX));
    }
    void launch_repel()
    {
        if (repulsion == FA2CU_REPULSION_BH) {
            launch_build();
            launch_sort();
            launch_tree();
        }
        launch_repulsion();
    }
    void launch_forces()
    {
        launch_repel();
        if (beside()) { // the iteration's order: repulsion + (gravity + attraction)
            launch_attraction_own(s, true);
            k_add_forces<R><<<ceil_div(n, 256), 256, 0, s>>>(n, fatt, f);
        } else {
            launch_attraction();
        }
    }
    // FP32 Barnes-Hut: gravity and attraction into fatt, on stream s2
    // beside the tree build and the walk, added to the repulsion by the
    // join (overlap 1: forked after the sort; 2: after the tree; 0: the
    // attraction fused with the totals after the walk). Forked after the
    // sort on one block per SM it measured 0.727 -> 0.711 ms an iteration at
    // 10^6 SBM nodes, 0.229 -> 0.209 ms at 10^5 BA nodes; forked before the
    // sort it delays the sort's tiles (0.77-0.85 ms, whatever the stream
    // priorities), and more blocks per SM slow the walk.
    bool beside() const { return overlap && s2 && fatt && !serial_totals<R>(n); }
    // alone: nothing runs beside it (the force query, the phase times), one
    // thread per node; else attract_grid blocks per SM
    void launch_attraction_own(cudaStream_t st, bool alone)
    {
        if constexpr (sizeof(R) == 4) {
            int sms = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
            if (nheavy > 0)
                k_attract_heavy<R, true><<<ceil_div(nheavy, 8), 256, 0, st>>>(
                    nheavy, heavy, linlog, adjust, pos, size, inc_off, inc, fatt);
            const int grid =
                alone ? ceil_div(n, 256)
                      : std::max(1, std::min(std::max(sms, 1) * attract_grid, ceil_div(n, 256)));
            k_attract_own<R><<<grid, 256, 0, st>>>(n, gravity, strong, linlog, adjust, pos, mass,
                                                   size, inc_off, inc, fatt);
        }
    }
    void launch_join_swing()
    {
        k_join_swing<R><<<std::min(ceil_div(n, 256), join_blocks), 256, 0, s>>>(
            n, fatt, f, fold, mass, fixed, sw, trac, swing_partial,
            (unsigned *) (status + ST_TICKET_SWING), st, status);
    }
    void launch_iteration()
    {
        if (beside()) {
            launch_build();
            launch_sort();
            if (overlap == 2) launch_tree();
            cudaEventRecord(ev_fork, s);
            cudaStreamWaitEvent(s2, ev_fork, 0);
            launch_attraction_own(s2, false);
            cudaEventRecord(ev_join, s2);
            if (overlap != 2) launch_tree();
            launch_repulsion();
            cudaStreamWaitEvent(s, ev_join, 0);
            launch_join_swing();
            launch_move();
            return;
        }
        launch_repel();
        launch_attraction_swing();
        launch_move();
    }

    int capture(cudaGraphExec_t *out, int iters)
    {
        cudaGraph_t g = nullptr;
        FA2_TRY(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal),
                "could not capture the iteration", 1);
        for (int k = 0; k < iters; k++) launch_iteration();
        cudaError_t e = cudaStreamEndCapture(s, &g);
        if (e != cudaSuccess) {
            set_cuda_error("could not capture the iteration", e);
            return 1;
        }
        if (iters == 1) { // the kernels of one iteration
            size_t nodes = 0;
            if (cudaGraphGetNodes(g, nullptr, &nodes) == cudaSuccess) {
                std::vector<cudaGraphNode_t> v(nodes);
                launches = 0;
                if (nodes && cudaGraphGetNodes(g, v.data(), &nodes) == cudaSuccess)
                    for (cudaGraphNode_t x : v) {
                        cudaGraphNodeType t;
                        if (cudaGraphNodeGetType(x, &t) == cudaSuccess &&
                            t == cudaGraphNodeTypeKernel)
                            launches++;
                    }
            }
        }
        e = cudaGraphInstantiate(out, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            set_cuda_error("could not instantiate the iteration graph", e);
            return 1;
        }
        return 0;
    }

    int iterate(int iterations) override
    {
        cudaSetDevice(device);
        while (iterations >= 8 && g8) {
            FA2_TRY(cudaGraphLaunch(g8, s), "the computation on the GPU failed", 1);
            iterations -= 8;
        }
        for (; iterations > 0; iterations--)
            FA2_TRY(cudaGraphLaunch(g1, s), "the computation on the GPU failed", 1);
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
        if (h & ERR_WAIT) {
            set_message("the computation on the GPU failed (a device wait timed out)");
            return 1;
        }
        if (h & ERR_BOUNDS) {
            set_message("the computation on the GPU failed (an index left its bounds)");
            return 1;
        }
        return 0;
    }

    int positions(double *out) override
    {
        cudaSetDevice(device);
        k_pos_out<R><<<ceil_div(n, 256), 256, 0, s>>>(n, pos, xy);
        FA2_TRY(cudaMemcpyAsync(out, xy, 2 * (size_t) n * sizeof(double),
                                cudaMemcpyDeviceToHost, s),
                "could not fetch the layout from the device", 1);
        FA2_TRY(cudaStreamSynchronize(s), "could not fetch the layout from the device", 1);
        return 0;
    }

    int set_positions(const double *in) override
    {
        cudaSetDevice(device);
        FA2_TRY(cudaMemcpyAsync(xy, in, 2 * (size_t) n * sizeof(double),
                                cudaMemcpyHostToDevice, s),
                "could not send the positions to the device", 1);
        k_pos_in<R><<<ceil_div(n, 256), 256, 0, s>>>(n, xy, pos);
        if (bbox_partial) launch_bbox();
        FA2_TRY(cudaStreamSynchronize(s), "could not send the positions to the device", 1);
        return 0;
    }

    int forces(const double *in, double *out) override
    {
        if (set_positions(in)) return 1;
        launch_forces();
        k_forces_out<R><<<ceil_div(n, 256), 256, 0, s>>>(n, f, nullptr, xy, xy + n);
        FA2_TRY(cudaMemcpyAsync(out, xy, 2 * (size_t) n * sizeof(double),
                                cudaMemcpyDeviceToHost, s),
                "could not fetch the forces", 1);
        return sync();
    }

    int speed(double state[4]) override
    {
        cudaSetDevice(device);
        SpeedState h;
        FA2_TRY(cudaMemcpyAsync(&h, st, sizeof(h), cudaMemcpyDeviceToHost, s), "cudaMemcpy", 1);
        FA2_TRY(cudaStreamSynchronize(s), "cudaMemcpy", 1);
        state[0] = h.speed;
        state[1] = h.efficiency;
        state[2] = h.total_swinging;
        state[3] = h.total_traction;
        return 0;
    }

    int phase_times(int iterations, double *ms) override
    {
        cudaSetDevice(device);
        for (int it = 0; it < iterations; it++) {
            int e = 0;
            cudaEventRecord(ev[e++], s);
            if (repulsion == FA2CU_REPULSION_BH) {
                launch_build();
                cudaEventRecord(ev[e++], s);
                launch_sort();
                cudaEventRecord(ev[e++], s);
                launch_tree();
                cudaEventRecord(ev[e++], s);
            } else {
                cudaEventRecord(ev[e++], s);
                cudaEventRecord(ev[e++], s);
                cudaEventRecord(ev[e++], s);
            }
            launch_repulsion();
            cudaEventRecord(ev[e++], s);
            if (beside()) { // "attraction": here after the walk, one thread per node, and the join
                launch_attraction_own(s, true);
                launch_join_swing();
            } else {
                launch_attraction_swing(); // with the totals and speed
            }
            cudaEventRecord(ev[e++], s);
            launch_move();
            cudaEventRecord(ev[e++], s);
            FA2_TRY(cudaEventSynchronize(ev[e - 1]), "the computation on the GPU failed", 1);
            double total = 0.0;
            for (int k = 1; k < e; k++) {
                float t = 0.f;
                cudaEventElapsedTime(&t, ev[k - 1], ev[k]);
                ms[k] += t;
                total += t;
            }
            ms[FA2_FULL_T_TOTAL] += total;
        }
        return sync();
    }

    int tree(const double *in, uint32_t *hkey, uint32_t *horder, int *hchild, int *hrange,
             int *hparent, double *hni) override
    {
        if (repulsion != FA2CU_REPULSION_BH) {
            set_message("this layout has no tree (exact repulsion)");
            return 1;
        }
        if (set_positions(in)) return 1;
        launch_build();
        launch_sort();
        launch_tree();
        std::vector<R4> hc((size_t) n - 1);
        std::vector<Agg<R>> ha(sizeof(R) == 4 ? (size_t) n - 1 : 0);
        const size_t nn = (size_t) n;
        cudaMemcpyAsync(hkey, key, nn * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(horder, order, nn * 4, cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hchild, child, (nn - 1) * sizeof(int2), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hrange, range, (nn - 1) * sizeof(int2), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hparent, parent, (2 * nn - 1) * sizeof(int), cudaMemcpyDeviceToHost, s);
        cudaMemcpyAsync(hc.data(), rec_c, (nn - 1) * sizeof(R4), cudaMemcpyDeviceToHost, s);
        if (sizeof(R) == 4)
            cudaMemcpyAsync(ha.data(), agg, (nn - 1) * sizeof(Agg<R>), cudaMemcpyDeviceToHost, s);
        FA2_TRY(cudaStreamSynchronize(s), "could not fetch the tree", 1);
        for (size_t r = 0; r + 1 < nn; r++) {
            hni[4 * r] = (double) hc[r].x;
            hni[4 * r + 1] = (double) hc[r].y;
            hni[4 * r + 2] = (double) hc[r].z;
            if (sizeof(R) == 4) { // the FP32 record holds a scaled size^2 (region_far)
                const float w = (float) (ha[r].maxx - ha[r].minx);
                const float h = (float) (ha[r].maxy - ha[r].miny);
                hni[4 * r + 3] = (double) (2.0f * (w * w + h * h));
            } else {
                hni[4 * r + 3] = (double) hc[r].w;
            }
        }
        return 0;
    }

    // The iteration graphs again, after an option changed the launches.
    int recapture()
    {
        cudaSetDevice(device);
        FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
        if (g1) cudaGraphExecDestroy(g1);
        if (g8) cudaGraphExecDestroy(g8);
        g1 = g8 = nullptr;
        if (capture(&g1, 1)) return 1;
        if (n <= (1 << 16) && capture(&g8, 8)) return 1;
        return 0;
    }

    int option(const char *name, double value) override
    {
        if (!strcmp(name, "sort_threads") && (value == 256 || value == 512 || value == 1024)) {
            ss.tile_threads = (int) value;
            return recapture();
        }
        if (!strcmp(name, "overlap") && (value == 0 || value == 1 || value == 2)) {
            if (value != 0 && !s2) {
                set_message("the attraction runs beside the walk in FP32 Barnes-Hut layouts only");
                return 1;
            }
            overlap = (int) value;
            return recapture();
        }
        if (!strcmp(name, "pdl") && (value == 0 || value == 1)) {
            pdl = value == 1;
            ss.pdl = pdl;
            return recapture();
        }
        if (!strcmp(name, "join_blocks") && value >= 1 && value <= 1 << 20) {
            join_blocks = (int) value;
            return recapture();
        }
        if (!strcmp(name, "attract_grid") && value >= 1 && value <= 8) {
            attract_grid = (int) value;
            return recapture();
        }
        if (!strcmp(name, "sort_block") && (value == 0 || value == 1)) {
            if (value == 1 && n > SORT_BLOCK_MAX) {
                set_message("the one-block sort handles at most %d keys", SORT_BLOCK_MAX);
                return 1;
            }
            block_sort = value == 1;
            return recapture();
        }
        if (!strcmp(name, "climb") &&
            (value == 1 || value == 2 || value == 4 || value == 8 || value == -2 ||
             value == -4)) {
            climb_mode = (int) value;
            return recapture();
        }
        if (!strcmp(name, "walk") &&
            (value == WALK_WARP || value == WALK_THREAD || value == WALK_THREAD_WIDE ||
             value == WALK_PAIR || value == WALK_QUAD || value == WALK_DEFERRED)) {
            walk = (int) value;
            return recapture();
        }
        if (!strcmp(name, "keep_traction") && value == 1) {
            // per-node traction kept for fa2cu_layout_swing (the FP64 path
            // keeps it anyway up to SERIAL_TOTALS_MAX nodes)
            if (!trac) {
                cudaSetDevice(device);
                FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
                trac = mem.get<R>((size_t) n);
                if (!trac) {
                    set_cuda_error("could not allocate memory on the device", mem.err);
                    return 1;
                }
            }
            return recapture();
        }
        set_message("unknown option %s = %g", name, value);
        return 1;
    }

    double info(const char *name) override
    {
        if (!strcmp(name, "launches_per_iteration")) return launches;
        if (!strcmp(name, "heavy_nodes")) return nheavy;
        if (!strcmp(name, "nodes")) return n;
        if (!strcmp(name, "incidences")) return ninc;
        set_message("unknown layout information %s", name);
        return -1.0;
    }

    int swing(double *hsw, double *htr) override
    {
        if (htr && !trac) {
            set_message("the per-node traction is not kept (option keep_traction)");
            return 1;
        }
        cudaSetDevice(device);
        std::vector<R> a((size_t) n), b(htr ? (size_t) n : 0);
        FA2_TRY(cudaMemcpyAsync(a.data(), sw, (size_t) n * sizeof(R), cudaMemcpyDeviceToHost, s),
                "could not fetch the swinging", 1);
        if (htr)
            FA2_TRY(cudaMemcpyAsync(b.data(), trac, (size_t) n * sizeof(R),
                                    cudaMemcpyDeviceToHost, s),
                    "could not fetch the traction", 1);
        FA2_TRY(cudaStreamSynchronize(s), "could not fetch the swinging", 1);
        for (int i = 0; i < n; i++) {
            if (hsw) hsw[i] = (double) a[i];
            if (htr) htr[i] = (double) b[i];
        }
        return 0;
    }

    int traversal_counts(double out[2]) override
    {
        if (repulsion != FA2CU_REPULSION_BH) {
            set_message("this layout has no tree (exact repulsion)");
            return 1;
        }
        cudaSetDevice(device);
        launch_build();
        launch_sort();
        launch_tree();
        cudaMemsetAsync(counts, 0, 2 * sizeof(unsigned long long), s);
        k_traverse_count<R><<<ceil_div(n, 256), 256, 0, s>>>(n, theta2, theta2d, psort, rec_c,
                                                             rec_t, agg, rope, counts);
        unsigned long long h[2] = {0, 0};
        cudaMemcpyAsync(h, counts, sizeof(h), cudaMemcpyDeviceToHost, s);
        FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
        out[0] = (double) h[0];
        out[1] = (double) h[1];
        return 0;
    }
};

template <class R>
LayoutBase *make_layout(const fa2_full_params *p, const double *pos, int rep,
                        const LayoutOpts *opts, const EdgeList *edges)
{
    int dev = p->device;
    FA2_TRY(cudaSetDevice(dev), "could not use the CUDA device", nullptr);
    Layout<R> *L = new Layout<R>();
    L->device = dev;
    if (L->open(p, pos, rep, opts, edges)) {
        delete L;
        return nullptr;
    }
    return L;
}

// Device bytes a layout holds (its buffers, counted by the allocation plan
// itself) plus the transient staging of the graph upload at open.
template <class R>
double layout_footprint(int n, int ninc, int adjust, int any_fixed, int rep, int sms)
{
    Layout<R> L;
    L.n = n;
    L.ninc = ninc;
    L.adjust = adjust ? 1 : 0;
    L.any_fixed = any_fixed ? 1 : 0;
    if (rep == FA2CU_REPULSION_EXACT)
        L.exact_nrows = exact_rows<R>(n, std::max(sms, 1), Layout<R>::EXACT_IPT);
    L.mem.dry = true;
    L.alloc(rep == FA2CU_REPULSION_BH);
    const double staging = (double) std::max(n, ninc) * sizeof(double) + (double) ninc * sizeof(int);
    return L.mem.bytes + staging;
}

// ---- the repulsion backend of fa2_gpu_open (reference src/gpu.c:357-704) --

template <class R> struct Repulse : RepulseBase {
    typedef typename RT<R>::R2 R2;
    typedef typename RT<R>::R4 R4;
    int n = 0, adjust = 0, barnes_hut = 0;
    cudaStream_t s = nullptr;
    DevMem mem;
    double *in4 = nullptr;   // x, y, mass, size staging (4n)
    double *out2 = nullptr;  // fx, fy (2n)
    double *host2 = nullptr; // pinned copy of out2
    R4 *p = nullptr;
    R2 *f = nullptr;
    R2 *part = nullptr; // partial sums of the split all-pairs kernel
    int nrows = 1;
    int *status = nullptr;
    fa2_region *raw = nullptr;
    QRegion<R> *regs = nullptr;
    int *perm = nullptr;

    ~Repulse() override
    {
        if (s) cudaStreamSynchronize(s);
        mem.release();
        if (host2) cudaFreeHost(host2);
        if (s) cudaStreamDestroy(s);
    }

    int open(int n_, int adjust_, int bh)
    {
        n = n_;
        adjust = adjust_ ? 1 : 0;
        barnes_hut = bh ? 1 : 0;
        const size_t nn = (size_t) n;
        FA2_TRY(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking),
                "could not create a CUDA stream", 1);
        in4 = mem.get<double>(4 * nn);
        out2 = mem.get<double>(2 * nn);
        p = mem.get<R4>(nn);
        f = mem.get<R2>(nn);
        status = mem.get<int>(ST_COUNT);
        if (!barnes_hut) {
            int sms = 0;
            cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
            nrows = exact_rows<R>(n, std::max(sms, 1), Layout<R>::EXACT_IPT);
            if (nrows > 1) part = mem.get<R2>((size_t) nrows * nn);
        }
        if (barnes_hut) {
            raw = mem.get<fa2_region>(2 * nn);
            regs = mem.get<QRegion<R>>(2 * nn);
            perm = mem.get<int>(nn);
        }
        if (mem.failed) {
            set_cuda_error("could not allocate memory on the device", mem.err);
            return 1;
        }
        FA2_TRY(cudaMallocHost(&host2, 2 * nn * sizeof(double)), "out of memory", 1);
        FA2_TRY(cudaMemsetAsync(status, 0, ST_COUNT * sizeof(int), s), "cudaMemset", 1);
        if (!barnes_hut) {
            const size_t smem = exact_smem_bytes<R>();
            FA2_TRY(cudaFuncSetAttribute(k_exact<R, false, Layout<R>::EXACT_IPT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem),
                    "cudaFuncSetAttribute", 1);
            FA2_TRY(cudaFuncSetAttribute(k_exact<R, true, Layout<R>::EXACT_IPT>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int) smem),
                    "cudaFuncSetAttribute", 1);
        }
        FA2_TRY(cudaStreamSynchronize(s), "could not prepare the device", 1);
        return 0;
    }

    int send4(const double *x, const double *y, const double *m, const double *sz)
    {
        const size_t b = (size_t) n * sizeof(double);
        FA2_TRY(cudaMemcpyAsync(in4, x, b, cudaMemcpyHostToDevice, s), "the computation on the GPU failed", 1);
        FA2_TRY(cudaMemcpyAsync(in4 + n, y, b, cudaMemcpyHostToDevice, s), "the computation on the GPU failed", 1);
        FA2_TRY(cudaMemcpyAsync(in4 + 2 * (size_t) n, m, b, cudaMemcpyHostToDevice, s), "the computation on the GPU failed", 1);
        const bool with_size = adjust && sz;
        if (with_size)
            FA2_TRY(cudaMemcpyAsync(in4 + 3 * (size_t) n, sz, b, cudaMemcpyHostToDevice, s),
                    "the computation on the GPU failed", 1);
        k_pack_host<R><<<ceil_div(n, 256), 256, 0, s>>>(
            n, in4, in4 + n, in4 + 2 * (size_t) n, with_size ? in4 + 3 * (size_t) n : nullptr, p);
        return 0;
    }

    int fetch_add(const int *dperm, double *dx, double *dy)
    {
        double t0 = now_s();
        k_forces_out<R><<<ceil_div(n, 256), 256, 0, s>>>(n, f, dperm, out2, out2 + n);
        FA2_TRY(cudaMemcpyAsync(host2, out2, 2 * (size_t) n * sizeof(double),
                                cudaMemcpyDeviceToHost, s),
                "the computation on the GPU failed", 1);
        FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
        for (int i = 0; i < n; i++) {
            dx[i] += host2[i];
            dy[i] += host2[n + i];
        }
        t_fetch += now_s() - t0;
        return 0;
    }

    int check_status()
    {
        int h = 0;
        FA2_TRY(cudaMemcpy(&h, status + ST_ERROR, sizeof(int), cudaMemcpyDeviceToHost),
                "the computation on the GPU failed", 1);
        if (h) {
            set_message(h & ERR_WAIT ? "the computation on the GPU failed (a device wait timed out)"
                                     : "the computation on the GPU failed (an index left its bounds)");
            return 1;
        }
        return 0;
    }

    int exact(const double *x, const double *y, const double *m, const double *sz,
              double sc, double *dx, double *dy) override
    {
        cudaSetDevice(device);
        double t0 = now_s();
        if (send4(x, y, m, sz)) return 1;
        FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
        double t1 = now_s();
        t_send += t1 - t0;
        launch_exact<R, Layout<R>::EXACT_IPT>(s, n, adjust, (R) sc, p, f, part, nrows, status);
        FA2_TRY(cudaGetLastError(), "the computation on the GPU failed", 1);
        FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
        if (check_status()) return 1;
        t_compute += now_s() - t1;
        return fetch_add(nullptr, dx, dy);
    }

    int bh(const fa2_tree *t, double sc, double theta, double *dx, double *dy) override
    {
        cudaSetDevice(device);
        if (check_quadtree(n, t)) return 1;
        double t0 = now_s();
        if (send4(t->px, t->py, t->pm, t->ps)) return 1;
        FA2_TRY(cudaMemcpyAsync(raw, t->reg, (size_t) t->nreg * sizeof(fa2_region),
                                cudaMemcpyHostToDevice, s),
                "the computation on the GPU failed", 1);
        FA2_TRY(cudaMemcpyAsync(perm, t->perm, (size_t) n * sizeof(int), cudaMemcpyHostToDevice, s),
                "the computation on the GPU failed", 1);
        k_qregions<R><<<ceil_div(t->nreg, 256), 256, 0, s>>>(t->nreg, raw, regs);
        FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
        double t1 = now_s();
        t_send += t1 - t0;
        const double theta2d = theta * theta;
        const R theta2 = (R) theta2d;
        const double *px = in4, *py = in4 + n; // the host's doubles, tree order
        if (adjust)
            k_qtraverse<R, true><<<ceil_div(n, 256), 256, 0, s>>>(
                n, (R) sc, theta2, theta2d, p, px, py, regs, raw, t->nreg, f, status);
        else
            k_qtraverse<R, false><<<ceil_div(n, 256), 256, 0, s>>>(
                n, (R) sc, theta2, theta2d, p, px, py, regs, raw, t->nreg, f, status);
        FA2_TRY(cudaGetLastError(), "the computation on the GPU failed", 1);
        FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
        if (check_status()) return 1;
        t_compute += now_s() - t1;
        return fetch_add(perm, dx, dy);
    }
};

template <class R> RepulseBase *make_repulse(int device, int n, int adjust, int bh)
{
    FA2_TRY(cudaSetDevice(device), "could not use the CUDA device", nullptr);
    Repulse<R> *g = new Repulse<R>();
    g->device = device;
    if (g->open(n, adjust, bh)) {
        delete g;
        return nullptr;
    }
    return g;
}

} // namespace fa2cu

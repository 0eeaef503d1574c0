// sort_tree.cuh -- the precision-independent step of the construction: the
// stable LSD radix sort of (Morton key, node) pairs (reference
// inst/opencl/pipeline.cl:132-188). The Karras tree is in karras.cuh.
//
// The sort makes one pass over the keys for the histograms of every digit,
// then one launch per 8-bit digit: each block ranks its tile of keys stably,
// learns the tile's offset inside every digit from its predecessors'
// published counts (decoupled look-back) and scatters.
#pragma once

#include "common.cuh"

namespace fa2cu {

// Keys per block of the sort: 256 threads x 8 keys.
constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 8;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;

// Auxiliary words of a sort: the 4 x 256 digit histograms, the 4 x 256
// digit bases, the tile tickets of the 4 passes, the arrival ticket of the
// histogram kernel.
constexpr int SORT_AUX_HIST = 0, SORT_AUX_BASE = 1024, SORT_AUX_TICKET = 2048,
              SORT_AUX_DONE = 2052, SORT_AUX = 2056;

// Scratch of a sort of n pairs: the ping-pong buffers, the look-back words
// of each pass (4 x 256 per tile) and the auxiliary words; `err` (may be
// null) receives ERR_WAIT if a look-back wait ever gives up.
struct SortScratch {
    uint32_t *key_b = nullptr, *val_b = nullptr; // n each
    uint32_t *counts = nullptr;                  // sort_scratch_counts(n)
    uint32_t *digit_total = nullptr;             // SORT_AUX
    int *err = nullptr;
    int tile_threads = 1024; // threads of a scatter block (tile = 8 keys each)
    bool pdl = false;        // scatter passes launched as programmatic dependents
};
size_t sort_scratch_counts(int n); // entries of `counts`

// Kernel attributes the sort needs on the current device; call before the
// first sort there (outside any stream capture). 0, or 1 with the message.
int sort_setup();

// Stable sort of key/val (n pairs) by key, 4 passes of 8 bits; the result is
// back in key / val. hist_ready: the digit histograms were already made by
// the kernel that produced the keys (sort_prepare, then hist_begin /
// hist_add / hist_end there); else the sort makes them.
void sort_pairs(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                const SortScratch &w, bool hist_ready = false);

// The same sort by a single block of 1024 threads (block_sort_pairs, four
// passes in one launch): for few keys, where the passes' launches and
// look-backs cost more than the work. Scratch: key_b / val_b of w.
constexpr int SORT_BLOCK_MAX = 4096;
void sort_pairs_block(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                      const SortScratch &w);

// Clears the histograms and tickets (before the histogram pass).
void sort_prepare(cudaStream_t s, const SortScratch &w);
// Look-back words the histogram pass clears, for n keys and `passes` digits.
size_t sort_status_words(int n, int passes);

// Stable LSD radix sort (4 passes of 8 bits) of n (key, value) pairs by key,
// by one block of W warps. Warp w owns the contiguous chunk
// [w C, min(n, (w+1) C)), C a multiple of 32, and reads it in rounds of 32 in
// order; per pass each warp counts its digits, the block turns the counts into
// offsets (digits in order, warps in order within a digit), and each warp
// scatters its chunk with ranks from lane matching. Ping-pong through kb / vb;
// the result is back in key / val.
template <int W>
__device__ void block_sort_pairs(int n, uint32_t *key, uint32_t *val, uint32_t *kb,
                                 uint32_t *vb, uint32_t (*cnt)[256], uint32_t *base)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int chunk = ((n + 32 * W - 1) / (32 * W)) * 32;
    const int lo = min(n, w * chunk), hi = min(n, lo + chunk);
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    for (int pass = 0; pass < 4; pass++) {
        const int shift = 8 * pass;
        for (int d = threadIdx.x; d < W * 256; d += blockDim.x) (&cnt[0][0])[d] = 0;
        __syncthreads();
        for (int b = lo; b < hi; b += 32) {
            const int i = b + lane;
            const bool valid = i < hi;
            const unsigned act = __ballot_sync(0xffffffffu, valid);
            if (valid) {
                const unsigned d = (key[i] >> shift) & 255u;
                const unsigned peers = match_digit8(act, d);
                if ((peers & lt) == 0) cnt[w][d] += __popc(peers);
            }
            __syncwarp();
        }
        __syncthreads();
        // per digit: exclusive prefix over the warps, then over the digits
        if (threadIdx.x < 256) {
            uint32_t run = 0;
            for (int ww = 0; ww < W; ww++) {
                const uint32_t c = cnt[ww][threadIdx.x];
                cnt[ww][threadIdx.x] = run;
                run += c;
            }
            base[threadIdx.x] = run;
        }
        __syncthreads();
        if (w == 0) { // 8 digits per lane
            uint32_t v[8], s = 0;
            for (int q = 0; q < 8; q++) {
                v[q] = base[lane * 8 + q];
                s += v[q];
            }
            uint32_t incl = s;
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t t = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += t;
            }
            uint32_t run = incl - s;
            for (int q = 0; q < 8; q++) {
                base[lane * 8 + q] = run;
                run += v[q];
            }
        }
        __syncthreads();
        if (threadIdx.x < 256)
            for (int ww = 0; ww < W; ww++) cnt[ww][threadIdx.x] += base[threadIdx.x];
        __syncthreads();
        for (int b = lo; b < hi; b += 32) {
            const int i = b + lane;
            const bool valid = i < hi;
            const unsigned act = __ballot_sync(0xffffffffu, valid);
            uint32_t k = 0, v = 0, prior = 0, cntp = 0, r = 0;
            unsigned d = 0;
            if (valid) {
                k = key[i];
                v = val[i];
                d = (k >> shift) & 255u;
                const unsigned peers = match_digit8(act, d);
                r = __popc(peers & lt);
                cntp = __popc(peers);
                prior = cnt[w][d];
            }
            __syncwarp();
            if (valid) {
                if (r == 0) cnt[w][d] = prior + cntp;
                const uint32_t at = prior + r;
                if (at < (uint32_t) n) { // always, for consistent counts
                    kb[at] = k;
                    vb[at] = v;
                }
            }
            __syncwarp();
        }
        __syncthreads();
        uint32_t *t = key;
        key = kb;
        kb = t;
        t = val;
        val = vb;
        vb = t;
    }
}

// Block-wide inclusive scan of one value per thread (blockDim.x <= 1024).
__device__ __forceinline__ uint32_t block_incl_scan(uint32_t v, uint32_t *warp_tot,
                                                    uint32_t *total)
{
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t t = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += t;
    }
    if (lane == 31) warp_tot[w] = v;
    __syncthreads();
    if (w == 0) {
        const int nw = blockDim.x >> 5;
        uint32_t s = lane < nw ? warp_tot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t t = __shfl_up_sync(0xffffffffu, s, o);
            if (lane >= o) s += t;
        }
        if (lane < nw) warp_tot[lane] = s;
        if (lane == nw - 1) *total = s;
    }
    __syncthreads();
    const uint32_t r = v + (w > 0 ? warp_tot[w - 1] : 0);
    __syncthreads();
    return r;
}

// The sort's histogram pass inside a kernel of SORT_THREADS threads per
// block: every block calls hist_begin (clears its per-warp counters and a
// share of the look-back words), hist_add per key it has, then hist_end (adds
// its counts to the global ones; the last block to finish turns them into
// digit bases). Every thread of every block must reach hist_begin and
// hist_end.
struct SortHistShared {
    uint32_t h[SORT_THREADS / 32][4][256];
    uint32_t wt[32];
    uint32_t tot;
    int last;
};

__device__ __forceinline__ void hist_begin(SortHistShared &S, uint32_t *status, size_t nstatus)
{
    for (int d = threadIdx.x; d < (SORT_THREADS / 32) * 4 * 256; d += SORT_THREADS)
        (&S.h[0][0][0])[d] = 0;
    for (size_t i = (size_t) blockIdx.x * SORT_THREADS + threadIdx.x; i < nstatus;
         i += (size_t) gridDim.x * SORT_THREADS)
        status[i] = 0u;
    __syncthreads();
}

__device__ __forceinline__ void hist_add(SortHistShared &S, uint32_t key, int passes)
{
    const int w = threadIdx.x >> 5;
    for (int p = 0; p < passes; p++) atomicAdd(&S.h[w][p][(key >> (8 * p)) & 255u], 1u);
}

__device__ __forceinline__ void hist_end(SortHistShared &S, int passes, uint32_t *aux)
{
    __syncthreads();
    for (int p = 0; p < passes; p++) {
        uint32_t c = 0;
        for (int ww = 0; ww < SORT_THREADS / 32; ww++) c += S.h[ww][p][threadIdx.x];
        if (c) atomicAdd(aux + SORT_AUX_HIST + p * 256 + threadIdx.x, c);
    }
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) S.last = atomicAdd(aux + SORT_AUX_DONE, 1u) == gridDim.x - 1;
    __syncthreads();
    if (!S.last) return;
    __threadfence();
    for (int p = 0; p < passes; p++) {
        const uint32_t c = __ldcg(aux + SORT_AUX_HIST + p * 256 + threadIdx.x);
        const uint32_t incl = block_incl_scan(c, S.wt, &S.tot);
        aux[SORT_AUX_BASE + p * 256 + threadIdx.x] = incl - c;
        aux[SORT_AUX_HIST + p * 256 + threadIdx.x] = 0u;
    }
    if (threadIdx.x < 4) aux[SORT_AUX_TICKET + threadIdx.x] = 0u;
    if (threadIdx.x == 0) aux[SORT_AUX_DONE] = 0u;
}

// The same with `passes` (1..4) passes of 8 bits, for keys below
// 2^(8 passes); the sorted pairs are left in (*kout, *vout), either key / val
// or the scratch buffers.
void sort_pairs_passes(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                       const SortScratch &w, int passes, uint32_t **kout, uint32_t **vout,
                       bool hist_ready = false);

} // namespace fa2cu

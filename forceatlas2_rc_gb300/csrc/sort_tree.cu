// sort_tree.cu -- stable LSD radix sort of (Morton key, node index) pairs and
// the Karras binary radix tree over the sorted keys.
//
// Sort (reference pipeline.cl:132-188 / src/gpu_full.c:419-435, four passes
// of 8 bits; any stable sort gives the reference's order, ties by index):
//   hist    per block of SORT_TILE keys, its 256 digit counts (shared-memory
//           counters fed by warp-aggregated increments: __match_any_sync
//           groups the lanes with equal digits, one lane adds the group);
//   scan    one block per digit: exclusive scan of that digit's counts over
//           the blocks, and the digit's total;
//   scatter each block ranks its keys stably with warp-ballot matching
//           (lanes in order, rounds in order, warps in order), stages them
//           by digit in shared memory, then writes runs of equal digits to
//           consecutive global positions.
#include "sort_tree.cuh"
#include "karras.cuh"

namespace fa2cu {

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

__global__ void __launch_bounds__(SORT_THREADS)
k_sort_hist(int n, int shift, const uint32_t *__restrict__ key, uint32_t *__restrict__ counts,
            int nb)
{
    __shared__ uint32_t h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int base = blockIdx.x * SORT_TILE;
    const int lane = threadIdx.x & 31;
#pragma unroll 4
    for (int it = 0; it < SORT_ITEMS; it++) {
        const int idx = base + it * SORT_THREADS + threadIdx.x;
        const bool valid = idx < n;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (valid) {
            const unsigned d = (key[idx] >> shift) & 255u;
            const unsigned peers = __match_any_sync(act, d);
            if ((peers & lanemask_lt()) == 0) atomicAdd(&h[d], (uint32_t) __popc(peers));
        }
        (void) lane;
    }
    __syncthreads();
    counts[threadIdx.x * nb + blockIdx.x] = h[threadIdx.x];
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

__global__ void __launch_bounds__(1024)
k_sort_scan(int nb, uint32_t *__restrict__ counts, uint32_t *__restrict__ digit_total)
{
    __shared__ uint32_t wt[32];
    __shared__ uint32_t tot;
    uint32_t *c = counts + (size_t) blockIdx.x * nb;
    uint32_t carry = 0;
    for (int base = 0; base < nb; base += blockDim.x) {
        const int i = base + threadIdx.x;
        const uint32_t v = i < nb ? c[i] : 0;
        const uint32_t incl = block_incl_scan(v, wt, &tot);
        if (i < nb) c[i] = carry + incl - v;
        carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) digit_total[blockIdx.x] = carry;
}

__global__ void __launch_bounds__(SORT_THREADS)
k_sort_scatter(int n, int shift, const uint32_t *__restrict__ kin, const uint32_t *__restrict__ vin,
               const uint32_t *__restrict__ counts, const uint32_t *__restrict__ digit_total,
               uint32_t *__restrict__ kout, uint32_t *__restrict__ vout, int nb)
{
    constexpr int NW = SORT_THREADS / 32;
    constexpr int PER_WARP = SORT_TILE / NW; // contiguous keys per warp
    constexpr int ROUNDS = PER_WARP / 32;
    __shared__ uint32_t wh[NW][256];
    __shared__ uint32_t lbase[256], gbase[256];
    __shared__ uint32_t wt[32];
    __shared__ uint32_t tot;
    __shared__ uint32_t sk[SORT_TILE], sv[SORT_TILE];

    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int d = threadIdx.x; d < NW * 256; d += SORT_THREADS) (&wh[0][0])[d] = 0;
    // global start of each digit: exclusive scan of the digit totals, plus
    // this block's offset inside the digit
    {
        const uint32_t t = digit_total[threadIdx.x];
        const uint32_t incl = block_incl_scan(t, wt, &tot);
        gbase[threadIdx.x] = incl - t + counts[threadIdx.x * nb + blockIdx.x];
    }
    __syncthreads();

    const int base = blockIdx.x * SORT_TILE + w * PER_WARP;
    uint32_t k[ROUNDS], v[ROUNDS];
    uint32_t rk[ROUNDS];
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        const int idx = base + r * 32 + lane;
        const bool valid = idx < n;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        k[r] = valid ? kin[idx] : 0u;
        v[r] = valid ? vin[idx] : 0u;
        uint32_t prior = 0, lt = 0, cnt = 0;
        unsigned d = (k[r] >> shift) & 255u;
        if (valid) {
            const unsigned peers = __match_any_sync(act, d);
            lt = __popc(peers & lanemask_lt());
            cnt = __popc(peers);
            prior = wh[w][d];
        }
        __syncwarp();
        if (valid && lt == 0) wh[w][d] = prior + cnt;
        __syncwarp();
        rk[r] = valid ? prior + lt : 0xffffffffu;
    }
    __syncthreads();
    // per digit: exclusive prefix over the warps, and the block's count
    {
        const int d = threadIdx.x;
        uint32_t run = 0;
#pragma unroll
        for (int ww = 0; ww < NW; ww++) {
            const uint32_t c = wh[ww][d];
            wh[ww][d] = run;
            run += c;
        }
        const uint32_t incl = block_incl_scan(run, wt, &tot);
        lbase[d] = incl - run;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        if (rk[r] == 0xffffffffu) continue;
        const unsigned d = (k[r] >> shift) & 255u;
        const uint32_t p = lbase[d] + wh[w][d] + rk[r];
        if (p < (uint32_t) SORT_TILE) { // always, for consistent counts
            sk[p] = k[r];
            sv[p] = v[r];
        }
    }
    __syncthreads();
    const int tile0 = blockIdx.x * SORT_TILE;
    const int cnt_tile = min(SORT_TILE, n - tile0);
    for (int i = threadIdx.x; i < cnt_tile; i += SORT_THREADS) {
        const uint32_t key = sk[i];
        const unsigned d = (key >> shift) & 255u;
        const uint32_t g = gbase[d] + (uint32_t) i - lbase[d];
        if (g < (uint32_t) n) { // always, for consistent counts
            kout[g] = key;
            vout[g] = sv[i];
        }
    }
}

size_t sort_scratch_counts(int n) { return 256 * (size_t) ceil_div(n, SORT_TILE); }

void sort_pairs_passes(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                       const SortScratch &w, int passes, uint32_t **kout, uint32_t **vout)
{
    const int nb = ceil_div(n, SORT_TILE);
    uint32_t *ka = key, *va = val, *kb = w.key_b, *vb = w.val_b;
    for (int pass = 0; pass < passes; pass++) {
        const int shift = 8 * pass;
        k_sort_hist<<<nb, SORT_THREADS, 0, s>>>(n, shift, ka, w.counts, nb);
        k_sort_scan<<<256, 1024, 0, s>>>(nb, w.counts, w.digit_total);
        k_sort_scatter<<<nb, SORT_THREADS, 0, s>>>(n, shift, ka, va, w.counts, w.digit_total,
                                                   kb, vb, nb);
        uint32_t *t = ka;
        ka = kb;
        kb = t;
        t = va;
        va = vb;
        vb = t;
    }
    *kout = ka;
    *vout = va;
}

void sort_pairs(cudaStream_t s, int n, uint32_t *key, uint32_t *val, const SortScratch &w)
{
    uint32_t *k = nullptr, *v = nullptr;
    sort_pairs_passes(s, n, key, val, w, 4, &k, &v); // four passes: back in key / val
}

// ---- Karras tree (pipeline.cl:209-270) -------------------------------------

__global__ void __launch_bounds__(256)
k_karras(int n, const uint32_t *__restrict__ key, int2 *__restrict__ child,
         int2 *__restrict__ range, int *__restrict__ parent, int *__restrict__ rope,
         int *__restrict__ visits)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n - 1) karras_one<true>(i, n, key, child, range, parent, rope, visits);
}

void karras_tree(cudaStream_t s, int n, const uint32_t *key, int2 *child, int2 *range,
                 int *parent, int *rope, int *visits)
{
    k_karras<<<ceil_div(n - 1, 256), 256, 0, s>>>(n, key, child, range, parent, rope, visits);
}

} // namespace fa2cu

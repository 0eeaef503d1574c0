// sort_tree.cu -- stable LSD radix sort of (Morton key, node index) pairs.
//
// Sort (reference pipeline.cl:132-188 / src/gpu_full.c:419-435, four passes
// of 8 bits; any stable sort gives the reference's order, ties by index):
//   hist4    one pass over the keys: the 256-bin histogram of every digit
//            (per-warp shared-memory counters, summed over the warps and
//            added to the global counts); the last block turns them into
//            digit bases (the Morton kernel does the same while it makes
//            the keys);
//   onesweep one launch per digit: each block takes the next tile of 8
//            keys per thread (256, 512 or 1024 threads), ranks them stably
//            (lanes, rounds and warps in order), publishes its per-digit
//            counts, adds those of the tiles before it (decoupled look-back,
//            bounded in time), stages the keys by digit in shared memory and
//            writes runs of equal digits to consecutive global positions;
//   block    up to a few thousand keys: one block sorts all four digits in
//            one launch (block_sort_pairs).
#include <algorithm>

#include "sort_tree.cuh"

namespace fa2cu {

__device__ __forceinline__ unsigned lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Histograms of every digit of the keys (one pass), the status words of the
// look-back zeroed; the last block to finish turns the histograms into digit
// bases (exclusive scans).
__global__ void __launch_bounds__(SORT_THREADS)
k_sort_hist4(int n, int passes, const uint32_t *__restrict__ key, uint32_t *__restrict__ status,
             size_t nstatus, uint32_t *__restrict__ aux)
{
    __shared__ SortHistShared S;
    hist_begin(S, status, nstatus);
    for (int idx = blockIdx.x * SORT_THREADS + threadIdx.x; idx < n;
         idx += gridDim.x * SORT_THREADS)
        hist_add(S, key[idx], passes);
    hist_end(S, passes, aux);
}

// Look-back words: the tile's count of a digit, or (once known) the count of
// every tile up to and including it.
constexpr uint32_t LB_COUNT = 1u << 30, LB_PREFIX = 1u << 31, LB_MASK = LB_COUNT - 1u;

__device__ __forceinline__ void lb_store(uint32_t *p, uint32_t v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ uint32_t lb_load(const uint32_t *p)
{
    uint32_t v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// One pass: each block takes the next tile of T * SORT_ITEMS keys (tickets
// in launch order, so a block only ever waits for tiles of blocks that
// started before it), ranks its keys stably (warp-contiguous chunks, lanes
// and rounds in order, warp matching), publishes its digit counts, adds its
// predecessors' (look-back: T/256 lookers per digit read 16 tiles each per
// round; bounded in time) and scatters through shared memory in runs of
// equal digits. Dynamic shared memory: per-warp digit counters, then the
// staged keys and values.
template <int T>
__global__ void __launch_bounds__(T)
k_sort_onesweep(int n, int pass, const uint32_t *__restrict__ kin,
                const uint32_t *__restrict__ vin, uint32_t *__restrict__ kout,
                uint32_t *__restrict__ vout, uint32_t *__restrict__ status,
                uint32_t *__restrict__ aux, int *__restrict__ err)
{
    constexpr int NW = T / 32;
    constexpr int TILE = T * SORT_ITEMS;
    constexpr int PER_WARP = TILE / NW; // contiguous keys per warp
    constexpr int ROUNDS = PER_WARP / 32;
    extern __shared__ __align__(16) uint32_t dsm[];
    uint32_t(*wh)[256] = reinterpret_cast<uint32_t(*)[256]>(dsm);
    uint32_t *sk = dsm + NW * 256, *sv = sk + TILE;
    __shared__ uint32_t lbase[256], gbase[256];
    __shared__ uint32_t wt[32];
    __shared__ uint32_t tot;
    __shared__ int tile_s;

    const int shift = 8 * pass;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    pdl_wait();
    if (threadIdx.x == 0) tile_s = (int) atomicAdd(aux + SORT_AUX_TICKET + pass, 1u);
    for (int d = threadIdx.x; d < NW * 256; d += T) dsm[d] = 0;
    __syncthreads();
    const int tile = tile_s;

    const int base = tile * TILE + w * PER_WARP;
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
            const unsigned peers = match_digit8(act, d);
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
    // per digit (threads 0..255): exclusive prefix over the warps and the
    // tile's count, published at once
    constexpr int W = T / 256; // lookers per digit
    __shared__ uint32_t lb_part[W][256];
    __shared__ int lb_stop[W][256]; // -2 all counts, -1 a prefix, else the unpublished tile
    __shared__ int lb_next[256];    // next tile to read back from (-1: done)
    __shared__ uint32_t lb_excl[256];
    const int dg = threadIdx.x & 255, looker = threadIdx.x >> 8;
    uint32_t run = 0;
    if (threadIdx.x < 256) {
#pragma unroll 8
        for (int ww = 0; ww < NW; ww++) {
            const uint32_t c = wh[ww][dg];
            wh[ww][dg] = run;
            run += c;
        }
        lb_store(status + (size_t) tile * 256 + dg, (tile == 0 ? LB_PREFIX : LB_COUNT) | run);
        lb_next[dg] = tile - 1;
        lb_excl[dg] = 0;
    }
    __syncthreads();
    // the look-back: each round, looker w of a digit reads the 16 tiles
    // from lb_next - 16w down (together W * 16 predecessors), summing counts
    // until it meets a prefix (done) or a word not yet published; the
    // digit's thread takes the windows in order, up to the first that did
    // not hold counts only, and goes on from an unpublished tile. Bounded in
    // time: after 1 s a digit gives up (error flag).
    const unsigned long long t0 = global_ns();
    bool gave_up = false;
    for (;;) {
        const int j0 = lb_next[dg];
        if (j0 >= 0) {
            const int jb = j0 - 16 * looker;
            uint32_t x[16];
#pragma unroll
            for (int q = 0; q < 16; q++)
                x[q] = jb - q >= 0 ? lb_load(status + (size_t) (jb - q) * 256 + dg) : LB_PREFIX;
            uint32_t sum = 0;
            int stop = -2;
#pragma unroll
            for (int q = 0; q < 16; q++) {
                if (stop != -2) continue;
                if (x[q] & (LB_PREFIX | LB_COUNT)) sum += x[q] & LB_MASK;
                if (x[q] & LB_PREFIX)
                    stop = -1;
                else if (!(x[q] & LB_COUNT))
                    stop = jb - q;
            }
            lb_part[looker][dg] = sum;
            lb_stop[looker][dg] = stop;
        }
        __syncthreads();
        bool more = false;
        if (threadIdx.x < 256 && j0 >= 0) {
            uint32_t e = lb_excl[dg];
            int next = j0 - 16 * W;
#pragma unroll
            for (int ww = 0; ww < W; ww++) {
                e += lb_part[ww][dg];
                const int st = lb_stop[ww][dg];
                if (st != -2) {
                    next = st; // -1 (done) or the tile to wait for
                    break;
                }
            }
            if (next >= 0 && global_ns() - t0 > 1000000000ull) {
                gave_up = true; // 1 s: a predecessor never published
                next = -1;
            }
            lb_excl[dg] = e;
            lb_next[dg] = next;
            more = next >= 0;
        }
        if (!__syncthreads_or(more)) break;
    }
    if (gave_up && err) atomicOr(err, ERR_WAIT);
    if (threadIdx.x < 256) {
        const uint32_t excl = lb_excl[dg];
        if (tile > 0) lb_store(status + (size_t) tile * 256 + dg, LB_PREFIX | ((excl + run) & LB_MASK));
        gbase[dg] = aux[SORT_AUX_BASE + pass * 256 + dg] + excl;
    }
    const uint32_t incl = block_incl_scan(run, wt, &tot); // threads >= 256 add 0
    if (threadIdx.x < 256) lbase[threadIdx.x] = incl - run;
    __syncthreads();
#pragma unroll
    for (int r = 0; r < ROUNDS; r++) {
        if (rk[r] == 0xffffffffu) continue;
        const unsigned d = (k[r] >> shift) & 255u;
        const uint32_t p = lbase[d] + wh[w][d] + rk[r];
        if (p < (uint32_t) TILE) { // always, for consistent counts
            sk[p] = k[r];
            sv[p] = v[r];
        }
    }
    __syncthreads();
    const int tile0 = tile * TILE;
    const int cnt_tile = min(TILE, n - tile0);
    for (int i = threadIdx.x; i < cnt_tile; i += T) {
        const uint32_t key = sk[i];
        const unsigned d = (key >> shift) & 255u;
        const uint32_t g = gbase[d] + (uint32_t) i - lbase[d];
        if (g < (uint32_t) n) { // always, for consistent counts
            kout[g] = key;
            vout[g] = sv[i];
        }
    }
}

template <int T> constexpr size_t onesweep_smem()
{
    return ((size_t) (T / 32) * 256 + 2 * (size_t) T * SORT_ITEMS) * sizeof(uint32_t);
}

int sort_setup()
{
    // the opt-in above 48 KB of dynamic shared memory of the larger tiles
    FA2_TRY(cudaFuncSetAttribute(k_sort_onesweep<512>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int) onesweep_smem<512>()),
            "cudaFuncSetAttribute", 1);
    FA2_TRY(cudaFuncSetAttribute(k_sort_onesweep<1024>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int) onesweep_smem<1024>()),
            "cudaFuncSetAttribute", 1);
    return 0;
}

template <int T>
static void onesweep_pass(cudaStream_t s, int n, int pass, const uint32_t *kin,
                          const uint32_t *vin, uint32_t *kout, uint32_t *vout,
                          const SortScratch &w)
{
    const int nb = ceil_div(n, T * SORT_ITEMS);
    launch_k(w.pdl, k_sort_onesweep<T>, dim3(nb), dim3(T), onesweep_smem<T>(), s, n, pass, kin,
             vin, kout, vout, w.counts + (size_t) pass * 256 * nb, w.digit_total, w.err);
}

__global__ void __launch_bounds__(1024)
k_sort_block(int n, uint32_t *__restrict__ key, uint32_t *__restrict__ val,
             uint32_t *__restrict__ kb, uint32_t *__restrict__ vb)
{
    __shared__ uint32_t cnt[32][256];
    __shared__ uint32_t base[256];
    block_sort_pairs<32>(n, key, val, kb, vb, cnt, base);
}

void sort_pairs_block(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                      const SortScratch &w)
{
    k_sort_block<<<1, 1024, 0, s>>>(n, key, val, w.key_b, w.val_b);
}

size_t sort_scratch_counts(int n) { return 4 * 256 * (size_t) ceil_div(n, SORT_TILE); }

size_t sort_status_words(int n, int passes) { return (size_t) passes * 256 * ceil_div(n, SORT_TILE); }

void sort_prepare(cudaStream_t s, const SortScratch &w)
{
    // histograms, bases and tickets start at zero
    cudaMemsetAsync(w.digit_total, 0, SORT_AUX * sizeof(uint32_t), s);
}

void sort_pairs_passes(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                       const SortScratch &w, int passes, uint32_t **kout, uint32_t **vout,
                       bool hist_ready)
{
    if (!hist_ready) {
        const int hist_blocks = std::min(ceil_div(n, SORT_TILE), 152 * 4);
        sort_prepare(s, w);
        k_sort_hist4<<<hist_blocks, SORT_THREADS, 0, s>>>(
            n, passes, key, w.counts, sort_status_words(n, passes), w.digit_total);
    }
    uint32_t *ka = key, *va = val, *kb = w.key_b, *vb = w.val_b;
    for (int pass = 0; pass < passes; pass++) {
        if (w.tile_threads == 1024)
            onesweep_pass<1024>(s, n, pass, ka, va, kb, vb, w);
        else if (w.tile_threads == 512)
            onesweep_pass<512>(s, n, pass, ka, va, kb, vb, w);
        else
            onesweep_pass<256>(s, n, pass, ka, va, kb, vb, w);
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

void sort_pairs(cudaStream_t s, int n, uint32_t *key, uint32_t *val, const SortScratch &w,
                bool hist_ready)
{
    uint32_t *k = nullptr, *v = nullptr;
    sort_pairs_passes(s, n, key, val, w, 4, &k, &v, hist_ready); // four passes: back in key / val
}

} // namespace fa2cu

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
    uint32_t *key_b, *val_b; // n each
    uint32_t *counts;        // sort_scratch_counts(n)
    uint32_t *digit_total;   // SORT_AUX
    int *err = nullptr;
    int tile_threads = 1024; // threads of a scatter block (tile = 8 keys each)
};
size_t sort_scratch_counts(int n); // entries of `counts`

// Kernel attributes the sort needs on the current device; call before the
// first sort there (outside any stream capture). 0, or 1 with the message.
int sort_setup();

// Stable sort of key/val (n pairs) by key, 4 passes of 8 bits; the result is
// back in key / val.
void sort_pairs(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                const SortScratch &w);

// The same with `passes` (1..4) passes of 8 bits, for keys below
// 2^(8 passes); the sorted pairs are left in (*kout, *vout), either key / val
// or the scratch buffers.
void sort_pairs_passes(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                       const SortScratch &w, int passes, uint32_t **kout, uint32_t **vout);

} // namespace fa2cu

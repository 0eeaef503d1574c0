// sort_tree.cuh -- precision-independent steps of the construction: the
// stable LSD radix sort of (Morton key, node) pairs and the Karras radix tree
// (reference inst/opencl/pipeline.cl:132-270).
#pragma once

#include "common.cuh"

namespace fa2cu {

// Keys per block of the sort: 256 threads x 8 keys.
constexpr int SORT_THREADS = 256;
constexpr int SORT_ITEMS = 8;
constexpr int SORT_TILE = SORT_THREADS * SORT_ITEMS;

// Scratch of a sort of n pairs: the ping-pong buffers and the per-block
// digit counts.
struct SortScratch {
    uint32_t *key_b, *val_b; // n each
    uint32_t *counts;        // 256 * nblocks
    uint32_t *digit_total;   // 256
};
size_t sort_scratch_counts(int n); // entries of `counts`

// Stable sort of key/val (n pairs) by key, 4 passes of 8 bits; the result is
// back in key / val.
void sort_pairs(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                const SortScratch &w);

// The same with `passes` (1..4) passes of 8 bits, for keys below
// 2^(8 passes); the sorted pairs are left in (*kout, *vout), either key / val
// or the scratch buffers.
void sort_pairs_passes(cudaStream_t s, int n, uint32_t *key, uint32_t *val,
                       const SortScratch &w, int passes, uint32_t **kout, uint32_t **vout);

// Karras tree over n >= 2 sorted keys: child[r] = (left, right),
// range[r] = (first, last) for the n-1 regions, parent of the 2n-1 tree nodes
// (leaves are n-1+k), rope[p] = right child of the region split after sorted
// node p (rope[n-1] = -1), visits reset to 0.
void karras_tree(cudaStream_t s, int n, const uint32_t *key, int2 *child, int2 *range,
                 int *parent, int *rope, int *visits);

} // namespace fa2cu

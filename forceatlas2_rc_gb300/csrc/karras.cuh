// karras.cuh -- one region of the Karras (2012) binary radix tree over
// sorted keys (reference inst/opencl/pipeline.cl:209-270), as a device
// function shared by the grid-wide build and the one-block-per-graph
// batched engine.
#pragma once

#include "common.cuh"

namespace fa2cu {

// Length of the common prefix of sorted keys i and j, -1 outside [0, n);
// equal keys are told apart by their indices. NC: the keys are read-only for
// the whole kernel (read through the non-coherent cache); false inside the
// batched engine, whose kernel also writes them.
template <bool NC>
__device__ __forceinline__ int cprefix(const uint32_t *key, int n, int i, uint32_t ki, int j)
{
    if (j < 0 || j >= n) return -1;
    const uint32_t kj = NC ? __ldg(key + j) : key[j];
    if (ki == kj) return 32 + __clz((unsigned) (i ^ j));
    return __clz(ki ^ kj);
}

// Region i (0 <= i < n-1) of the tree over n >= 2 sorted keys: its children
// (regions < n-1, leaves n-1+k), its range of sorted nodes, the parent links
// of its children, the rope entry of its split (the right child: the next
// region after the subtree that ends at the split), and its arrival counter.
template <bool NC>
__device__ __forceinline__ void karras_one(int i, int n, const uint32_t *key, int2 *child,
                                           int2 *range, int *parent, int *rope, int *visits)
{
    const uint32_t ki = NC ? __ldg(key + i) : key[i];
    const int d = cprefix<NC>(key, n, i, ki, i + 1) > cprefix<NC>(key, n, i, ki, i - 1) ? 1 : -1;
    const int pmin = cprefix<NC>(key, n, i, ki, i - d);
    int lmax = 2;
    while (cprefix<NC>(key, n, i, ki, i + lmax * d) > pmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
        if (cprefix<NC>(key, n, i, ki, i + (l + t) * d) > pmin) l += t;
    const int j = i + l * d;
    const int pnode = cprefix<NC>(key, n, i, ki, j);
    int s = 0, t = l;
    do {
        t = (t + 1) >> 1;
        if (cprefix<NC>(key, n, i, ki, i + (s + t) * d) > pnode) s += t;
    } while (t > 1);
    const int split = i + s * d + min(d, 0);
    const int first = min(i, j), last = max(i, j);
    const int left = first == split ? n - 1 + split : split;
    const int right = last == split + 1 ? n - 1 + split + 1 : split + 1;
    child[i] = make_int2(left, right);
    range[i] = make_int2(first, last);
    parent[left] = i;
    parent[right] = i;
    rope[split] = right;
    visits[i] = 0;
    if (i == 0) {
        parent[0] = -1;
        rope[n - 1] = -1;
    }
}

} // namespace fa2cu

// prep.cuh -- the graph's preparation on the device (prep.cu): masses and
// symmetric incidence lists from the edge list.
#pragma once

#include <algorithm>

#include "common.cuh"
#include "devmem.cuh"
#include "sort_tree.cuh"

namespace fa2cu {

struct PrepScratch {
    unsigned *deg = nullptr, *cnt = nullptr, *tile_sum = nullptr;
    int *bad = nullptr;
    uint32_t *key = nullptr, *val = nullptr;
    SortScratch sort{};
};

// Scratch of a preparation of n nodes and m edges, from `mem`.
void prep_scratch(DevMem &mem, int n, int m, PrepScratch &ws);
double prep_scratch_bytes(int n, int m);

// On stream s, from device arrays from / to (m ints) and w (m doubles):
// mass (n doubles), inc_off (n + 1 ints), inc_node / inc_coef (at most 2m
// entries). Returns the number of incidences, or -1 with the message set
// (an edge whose end is not a node: "edge %d refers to a node that does not
// exist", numbered from 1, the first such edge). Synchronises s twice.
long long prep_graph(cudaStream_t s, int n, int m, const int *from, const int *to,
                     const double *w, int outbound, double *mass, int *inc_off, int *inc_node,
                     double *inc_coef, const PrepScratch &ws);

} // namespace fa2cu

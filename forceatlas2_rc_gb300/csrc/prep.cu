// prep.cu -- the graph's preparation on the device: masses (1 + degree) and
// the symmetric incidence lists with their attraction coefficients, as
// C_forceatlas2_large builds them on the host (reference
// src/forceatlas2.c:868-902), from the edge list.
//
//   count   per edge: both ends' degrees (a self-loop counts twice), both
//           ends' incidence counts (self-loops have none), and the first
//           edge whose end is not a node;
//   offsets exclusive scan of the incidence counts (inc_off, n + 1);
//   keys    two entries per edge, (owner, 2e + side) with side 0 for the
//           source's entry and 1 for the target's; a self-loop's owner is n,
//           after every node;
//   sort    stable LSD radix sort by owner (as many 8-bit passes as n
//           needs): each node's incidences come out in edge order, the
//           order in which the reference appends them;
//   fill    the other end and the coefficient, in double:
//           coef * w[e] (/ mass[from[e]] with dissuade_hubs), coef the mean
//           mass (n + 2m) / n with dissuade_hubs, else 1.
//
// Masses are integers and their total is exactly n + 2m, so the mean is one
// correctly rounded division, as the reference's serial sum gives.
#include "prep.cuh"

namespace fa2cu {

__global__ void __launch_bounds__(256)
k_prep_count(int n, int m, const int *__restrict__ from, const int *__restrict__ to,
             unsigned *__restrict__ deg, unsigned *__restrict__ cnt, int *__restrict__ bad)
{
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x) {
        const int a = from[e], b = to[e];
        if ((unsigned) a >= (unsigned) n || (unsigned) b >= (unsigned) n) {
            atomicMin(bad, e);
            continue;
        }
        atomicAdd(deg + a, 1u);
        atomicAdd(deg + b, 1u);
        if (a != b) {
            atomicAdd(cnt + a, 1u);
            atomicAdd(cnt + b, 1u);
        }
    }
}

// Exclusive scan, phase 1: each block scans PREP_SCAN_TILE counts (4 per
// thread) in place and writes its total.
constexpr int PREP_SCAN_THREADS = 256;
constexpr int PREP_SCAN_TILE = 4 * PREP_SCAN_THREADS;

__global__ void __launch_bounds__(PREP_SCAN_THREADS)
k_prep_scan_tiles(int n, const unsigned *__restrict__ cnt, int *__restrict__ off,
                  unsigned *__restrict__ tile_sum)
{
    __shared__ unsigned wsum[PREP_SCAN_THREADS / 32];
    const int base = blockIdx.x * PREP_SCAN_TILE + 4 * threadIdx.x;
    unsigned v[4], s = 0;
    for (int q = 0; q < 4; q++) {
        v[q] = base + q < n ? cnt[base + q] : 0u;
        s += v[q];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned incl = s;
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += t;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    unsigned before = 0;
    for (int k = 0; k < w; k++) before += wsum[k];
    unsigned run = before + incl - s;
    for (int q = 0; q < 4; q++) {
        if (base + q < n) off[base + q] = (int) run;
        run += v[q];
    }
    if (threadIdx.x == PREP_SCAN_THREADS - 1) tile_sum[blockIdx.x] = run;
}

// Phase 2 (one block): exclusive scan of the tile totals; off[n] = total.
__global__ void __launch_bounds__(1024)
k_prep_scan_sums(int ntiles, int n, unsigned *__restrict__ tile_sum, int *__restrict__ off)
{
    __shared__ unsigned wsum[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int b0 = 0; b0 < ntiles; b0 += blockDim.x) {
        const int i = b0 + threadIdx.x;
        const unsigned v = i < ntiles ? tile_sum[i] : 0u;
        unsigned incl = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o) incl += t;
        }
        if (lane == 31) wsum[w] = incl;
        __syncthreads();
        unsigned before = 0;
        for (int k = 0; k < w; k++) before += wsum[k];
        if (i < ntiles) tile_sum[i] = carry + before + incl - v;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry += before + incl;
        __syncthreads();
    }
    if (threadIdx.x == 0) off[n] = (int) carry;
}

// Phase 3: add each tile's offset.
__global__ void __launch_bounds__(PREP_SCAN_THREADS)
k_prep_scan_add(int n, const unsigned *__restrict__ tile_sum, int *__restrict__ off)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) off[i] += (int) tile_sum[i / PREP_SCAN_TILE];
}

__global__ void __launch_bounds__(256)
k_prep_keys(int n, int m, const int *__restrict__ from, const int *__restrict__ to,
            const unsigned *__restrict__ deg, double *__restrict__ mass,
            uint32_t *__restrict__ key, uint32_t *__restrict__ val)
{
    const int stride = gridDim.x * blockDim.x;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += stride) {
        const int a = from[e], b = to[e];
        const bool loop = a == b;
        key[2 * (size_t) e] = loop ? (uint32_t) n : (uint32_t) a;
        key[2 * (size_t) e + 1] = loop ? (uint32_t) n : (uint32_t) b;
        val[2 * (size_t) e] = 2u * (uint32_t) e;
        val[2 * (size_t) e + 1] = 2u * (uint32_t) e + 1u;
    }
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
        mass[i] = 1.0 + (double) deg[i];
}

__global__ void __launch_bounds__(256)
k_prep_fill(const int *__restrict__ ntot, const int *__restrict__ from,
            const int *__restrict__ to, const double *__restrict__ w,
            const double *__restrict__ mass, int outbound, double coef,
            const uint32_t *__restrict__ val, int *__restrict__ inc_node,
            double *__restrict__ inc_coef)
{
    const int total = *ntot;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < total;
         k += gridDim.x * blockDim.x) {
        const uint32_t v = val[k];
        const int e = (int) (v >> 1);
        const int a = from[e], b = to[e];
        inc_node[k] = (v & 1u) ? a : b;
        const double c = __dmul_rn(coef, w[e]);
        inc_coef[k] = outbound ? __ddiv_rn(c, mass[a]) : c;
    }
}

void prep_scratch(DevMem &mem, int n, int m, PrepScratch &ws)
{
    const size_t two_m = 2 * (size_t) std::max(m, 1);
    ws.deg = mem.get<unsigned>((size_t) n);
    ws.cnt = mem.get<unsigned>((size_t) n);
    ws.tile_sum = mem.get<unsigned>((size_t) ceil_div(n, PREP_SCAN_TILE));
    ws.bad = mem.get<int>(1);
    ws.key = mem.get<uint32_t>(two_m);
    ws.val = mem.get<uint32_t>(two_m);
    ws.sort.key_b = mem.get<uint32_t>(two_m);
    ws.sort.val_b = mem.get<uint32_t>(two_m);
    ws.sort.counts = mem.get<uint32_t>(sort_scratch_counts((int) two_m));
    ws.sort.digit_total = mem.get<uint32_t>(SORT_AUX);
}

double prep_scratch_bytes(int n, int m)
{
    DevMem mem;
    mem.dry = true;
    PrepScratch ws;
    prep_scratch(mem, n, m, ws);
    return mem.bytes;
}

long long prep_graph(cudaStream_t s, int n, int m, const int *from, const int *to,
                     const double *w, int outbound, double *mass, int *inc_off, int *inc_node,
                     double *inc_coef, const PrepScratch &ws)
{
    const int big = 0x7fffffff;
    FA2_TRY(cudaMemsetAsync(ws.deg, 0, (size_t) n * sizeof(unsigned), s), "cudaMemset", -1);
    FA2_TRY(cudaMemsetAsync(ws.cnt, 0, (size_t) n * sizeof(unsigned), s), "cudaMemset", -1);
    FA2_TRY(cudaMemcpyAsync(ws.bad, &big, sizeof(int), cudaMemcpyHostToDevice, s), "cudaMemcpy",
            -1);
    const int grid_m = std::max(1, std::min(ceil_div(m, 256), 152 * 16));
    if (m > 0) k_prep_count<<<grid_m, 256, 0, s>>>(n, m, from, to, ws.deg, ws.cnt, ws.bad);
    int bad = big;
    FA2_TRY(cudaMemcpyAsync(&bad, ws.bad, sizeof(int), cudaMemcpyDeviceToHost, s), "cudaMemcpy",
            -1);
    FA2_TRY(cudaStreamSynchronize(s), "the graph preparation on the GPU failed", -1);
    if (bad != big) {
        set_message("edge %d refers to a node that does not exist", bad + 1);
        return -1;
    }
    const int ntiles = ceil_div(n, PREP_SCAN_TILE);
    k_prep_scan_tiles<<<ntiles, PREP_SCAN_THREADS, 0, s>>>(n, ws.cnt, inc_off, ws.tile_sum);
    k_prep_scan_sums<<<1, 1024, 0, s>>>(ntiles, n, ws.tile_sum, inc_off);
    k_prep_scan_add<<<ceil_div(n, PREP_SCAN_THREADS), PREP_SCAN_THREADS, 0, s>>>(n, ws.tile_sum,
                                                                                 inc_off);
    const int grid_nm = std::max(1, std::min(ceil_div(std::max(n, m), 256), 152 * 16));
    k_prep_keys<<<grid_nm, 256, 0, s>>>(n, m, from, to, ws.deg, mass, ws.key, ws.val);
    if (m > 0) {
        // 8-bit passes enough for owners 0 .. n
        int passes = 1;
        while (passes < 4 && ((uint64_t) n >> (8 * passes)) != 0) passes++;
        uint32_t *k = ws.key, *v = ws.val;
        if (sort_setup()) return -1;
        sort_pairs_passes(s, 2 * m, k, v, ws.sort, passes, &k, &v);
        const double mean = (double) ((long long) n + 2LL * (long long) m) / (double) n;
        k_prep_fill<<<std::max(1, std::min(ceil_div(2 * m, 256), 152 * 16)), 256, 0, s>>>(
            inc_off + n, from, to, w, mass, outbound, outbound ? mean : 1.0, v, inc_node,
            inc_coef);
    }
    int hn = 0;
    FA2_TRY(cudaMemcpyAsync(&hn, inc_off + n, sizeof(int), cudaMemcpyDeviceToHost, s),
            "cudaMemcpy", -1);
    FA2_TRY(cudaStreamSynchronize(s), "the graph preparation on the GPU failed", -1);
    return hn;
}

} // namespace fa2cu

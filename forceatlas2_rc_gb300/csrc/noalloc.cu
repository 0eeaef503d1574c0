// noalloc.cu -- the one entry point of libfa2cuda.so that allocates nothing:
// Morton codes and the stable Morton order of n nodes whose positions are
// already on the device (the first steps of the Barnes-Hut tree build),
// with every byte of scratch memory in a static device array of this file.
//
// It is for callers that cannot call cudaMalloc: a program whose device
// memory belongs to another allocator (a framework's memory pool that has to
// account for every byte on the GPU), or a code path that must neither wait
// for an allocation (cudaMalloc can synchronise the device) nor risk one
// failing once it has started. They pass device buffers for the input and
// the outputs; the sort's ping-pong buffers, its digit counts and the
// bounding-box partials live in g_scratch.
//
// Limits and sharing:
//   - at most NOALLOC_MAX_N = 2^20 nodes; larger n is rejected with a
//     message, nothing launched;
//   - g_scratch (about 9 MB) exists on every GPU that loads the library and
//     stays there until the process exits;
//   - every call shares it and it keeps the last call's contents: calls that
//     overlap on the GPU (on different streams, or from several host
//     threads) race and must not be issued; calls in one stream are fine;
//   - the first call on a device looks up the array's device address there
//     (cudaGetSymbolAddress, once per device, with that device current); that
//     first call should come before any stream capture.
#include <algorithm>

#include "kernels.cuh"
#include "sort_tree.cuh"

namespace fa2cu {

constexpr int NOALLOC_MAX_N = 1 << 20;
constexpr int NOALLOC_NB = NOALLOC_MAX_N / SORT_TILE; // sort blocks at the maximum
constexpr int NOALLOC_NBBOX = 152 * 4;                // bounding-box blocks

constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t OFF_KEY_B = 0;
constexpr size_t OFF_VAL_B = OFF_KEY_B + align256((size_t) NOALLOC_MAX_N * 4);
constexpr size_t OFF_COUNTS = OFF_VAL_B + align256((size_t) NOALLOC_MAX_N * 4);
constexpr size_t OFF_TOTAL = OFF_COUNTS + align256(4 * 256 * (size_t) NOALLOC_NB * 4);
constexpr size_t OFF_PART = OFF_TOTAL + align256(SORT_AUX * 4);
constexpr size_t OFF_BBOX = OFF_PART + align256(4 * (size_t) NOALLOC_NBBOX * 4);
constexpr size_t OFF_QUANT = OFF_BBOX + align256(4 * 4);
constexpr size_t OFF_TICKET = OFF_QUANT + align256(6 * 8);
constexpr size_t NOALLOC_BYTES = OFF_TICKET + align256(4);

// The scratch memory of fa2cu_morton_order_noalloc (one copy per device).
static __device__ __align__(256) unsigned char g_scratch[NOALLOC_BYTES];

// Device address of g_scratch on each device, looked up on first use there.
constexpr int NOALLOC_MAX_DEVICES = 64;
static unsigned char *g_scratch_addr[NOALLOC_MAX_DEVICES];

} // namespace fa2cu

using namespace fa2cu;

extern "C" int fa2cu_morton_order_noalloc(int n, const float *pos, uint32_t *key,
                                          uint32_t *order, void *stream)
{
    if (n < 1 || n > NOALLOC_MAX_N) {
        set_message("fa2cu_morton_order_noalloc handles 1 to %d nodes, not %d", NOALLOC_MAX_N,
                    n);
        return 1;
    }
    if (!pos || !key || !order) {
        set_message("fa2cu_morton_order_noalloc: invalid (NULL) device buffer");
        return 1;
    }
    int dev = 0;
    FA2_TRY(cudaGetDevice(&dev), "no current CUDA device", 1);
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        set_message("fa2cu_morton_order_noalloc supports devices 0 to %d", NOALLOC_MAX_DEVICES - 1);
        return 1;
    }
    if (!g_scratch_addr[dev]) {
        // host code may not use g_scratch itself: its name stands for a host
        // shadow, not the device array; take the device address once
        void *p = nullptr;
        FA2_TRY(cudaGetSymbolAddress(&p, g_scratch), "could not locate the scratch memory", 1);
        g_scratch_addr[dev] = (unsigned char *) p;
    }
    unsigned char *base = g_scratch_addr[dev];
    cudaStream_t s = (cudaStream_t) stream;
    unsigned *ticket = (unsigned *) (base + OFF_TICKET);
    // the last call may have left anything here: the arrival ticket of the
    // bounding-box reduction must start at zero (everything else is fully
    // written before it is read)
    FA2_TRY(cudaMemsetAsync(ticket, 0, sizeof(unsigned), s), "the computation on the GPU failed",
            1);
    const int nbbox = std::min(ceil_div(n, 256), NOALLOC_NBBOX);
    const float2 *p2 = reinterpret_cast<const float2 *>(pos);
    k_bbox<float><<<nbbox, 256, 0, s>>>(n, p2, (float *) (base + OFF_PART),
                                        (float *) (base + OFF_BBOX), (double *) (base + OFF_QUANT),
                                        ticket);
    k_morton<float><<<ceil_div(n, 256), 256, 0, s>>>(n, p2, (const double *) (base + OFF_QUANT),
                                                     key, order, nullptr, nullptr, 0);
    if (sort_setup()) return 1;
    SortScratch w;
    w.key_b = (uint32_t *) (base + OFF_KEY_B);
    w.val_b = (uint32_t *) (base + OFF_VAL_B);
    w.counts = (uint32_t *) (base + OFF_COUNTS);
    w.digit_total = (uint32_t *) (base + OFF_TOTAL);
    sort_pairs(s, n, key, order, w);
    FA2_TRY(cudaGetLastError(), "the computation on the GPU failed", 1);
    return 0;
}

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
//     (cudaGetSymbolAddress, once per device, with that device current). With
//     CUDA's default lazy module loading, that first lookup is also when the
//     library's device code and the array are loaded onto the device: it may
//     allocate and synchronise, so make it up front (fa2cu_noalloc_status
//     does only the lookup), before any stream capture;
//   - a look-back wait of the sort that gives up (after about a second; it
//     only happens if the GPU fails to run the sort's blocks) leaves key and
//     order wrong; the call itself returns before the GPU runs, so it cannot
//     say so: the error word in the array records it, and
//     fa2cu_noalloc_status reads it back once the stream is done.
#include <algorithm>
#include <atomic>
#include <cstdint>

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
// the bounding box's arrival ticket and the sort's error word, side by side
// so that one clear of 8 bytes starts both at zero
constexpr size_t OFF_TICKET = OFF_QUANT + align256(6 * 8);
constexpr size_t OFF_ERR = OFF_TICKET + 4;
constexpr size_t NOALLOC_BYTES = OFF_TICKET + align256(8);

// The scratch memory of fa2cu_morton_order_noalloc (one copy per device).
static __device__ __align__(256) unsigned char g_scratch[NOALLOC_BYTES];

// Device address of g_scratch on each device, looked up on first use there
// (atomic: host threads may make their first calls at the same time; they
// look up the same address).
constexpr int NOALLOC_MAX_DEVICES = 64;
static std::atomic<unsigned char *> g_scratch_addr[NOALLOC_MAX_DEVICES];

// g_scratch's address on the current device (looked up once), or null with
// the message set.
static unsigned char *scratch_base(const char *who)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) {
        cudaGetLastError();
        set_message("%s: no current CUDA device", who);
        return nullptr;
    }
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) {
        set_message("%s supports devices 0 to %d", who, NOALLOC_MAX_DEVICES - 1);
        return nullptr;
    }
    unsigned char *base = g_scratch_addr[dev].load(std::memory_order_acquire);
    if (!base) {
        // host code may not use g_scratch itself: its name stands for a host
        // shadow, not the device array; take the device address once
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
        if (e != cudaSuccess || !p) {
            cudaGetLastError();
            set_cuda_error("could not locate the scratch memory", e);
            return nullptr;
        }
        base = (unsigned char *) p;
        g_scratch_addr[dev].store(base, std::memory_order_release);
    }
    return base;
}

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
    // the kernels read pos as float2 and write key / order as 32-bit words:
    // a misaligned buffer would fault on the GPU, so it is refused here
    if (((uintptr_t) pos & 7) || ((uintptr_t) key & 3) || ((uintptr_t) order & 3)) {
        set_message("fa2cu_morton_order_noalloc: pos must be 8-byte aligned and key, order "
                    "4-byte aligned");
        return 1;
    }
    unsigned char *base = scratch_base("fa2cu_morton_order_noalloc");
    if (!base) return 1;
    cudaStream_t s = (cudaStream_t) stream;
    unsigned *ticket = (unsigned *) (base + OFF_TICKET);
    // the last call may have left anything here: the arrival ticket of the
    // bounding-box reduction and the sort's error word must start at zero
    // (everything else is fully written before it is read)
    FA2_TRY(cudaMemsetAsync(ticket, 0, 8, s), "the computation on the GPU failed", 1);
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
    w.err = (int *) (base + OFF_ERR);
    sort_pairs(s, n, key, order, w);
    FA2_TRY(cudaGetLastError(), "the computation on the GPU failed", 1);
    return 0;
}

extern "C" int fa2cu_noalloc_status(void *stream)
{
    unsigned char *base = scratch_base("fa2cu_noalloc_status");
    if (!base) return 1;
    cudaStream_t s = (cudaStream_t) stream;
    int err = 0;
    // ordered after the stream's earlier work, i.e. after the last call's sort
    FA2_TRY(cudaMemcpyAsync(&err, base + OFF_ERR, sizeof(int), cudaMemcpyDeviceToHost, s),
            "the computation on the GPU failed", 1);
    FA2_TRY(cudaStreamSynchronize(s), "the computation on the GPU failed", 1);
    if (err & ERR_WAIT) {
        set_message("the computation on the GPU failed (a device wait timed out): "
                    "the Morton order of the last call is wrong");
        return 1;
    }
    return 0;
}

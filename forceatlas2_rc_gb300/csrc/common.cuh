// common.cuh -- shared definitions of libfa2cuda.so: error reporting, the
// real-number traits of the two precisions, device helpers.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/fa2.h"
#include "../../include/fa2_cuda.h"

namespace fa2cu {

// ---- errors (the fa2_gpu_error() buffer, reference src/gpu.c:129-143) ----
void set_message(const char *fmt, ...);
void set_cuda_error(const char *what, cudaError_t e);
// The CUDA call of the expression, on failure: message and return `ret`.
#define FA2_TRY(expr, what, ret)                                               \
    do {                                                                       \
        cudaError_t e_ = (expr);                                               \
        if (e_ != cudaSuccess) {                                               \
            ::fa2cu::set_cuda_error(what, e_);                                 \
            return ret;                                                        \
        }                                                                      \
    } while (0)

// Barnes-Hut walk variants (all give identical forces): warp-synchronous;
// one walk per thread at 8 blocks of 256 per SM (<= 32 registers; 6 and <= 40
// with prevent_overlap or in double); one walk
// per thread with the registers the compiler wants; one thread walking for
// two or four Morton neighbours at once.
enum {
    WALK_WARP = 0,
    WALK_THREAD = 1,
    WALK_THREAD_WIDE = 2,
    WALK_PAIR = 3,
    WALK_QUAD = 4,
    WALK_DEFERRED = 5,
};

// Programmatic dependent launch. A kernel of the iteration may be launched
// with the programmatic stream serialisation attribute (launch_k): its
// blocks are then scheduled as its predecessor on the stream finishes,
// without a launch gap. It calls pdl_wait before touching memory: the wait
// returns once the predecessor grid has completed and its writes are
// visible (at once for a kernel launched without the attribute). No kernel
// triggers its dependents early, so a waiting block never holds an SM its
// predecessor still needs.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block,
                            size_t smem, cudaStream_t s, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = pdl ? attr : nullptr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, ((KArgs) args)...);
}

// Nanoseconds of the GPU's global timer (bounds of every device-side wait).
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// The lanes of `act` whose 8-bit digit equals this lane's: eight ballots,
// one per bit (the same mask as __match_any_sync, at ballot throughput).
// Every lane of `act` must call it.
__device__ __forceinline__ unsigned match_digit8(unsigned act, unsigned d)
{
    unsigned peers = act;
#pragma unroll
    for (int b = 0; b < 8; b++) {
        const bool bit = (d >> b) & 1u;
        const unsigned m = __ballot_sync(act, bit);
        peers &= bit ? m : ~m;
    }
    return peers;
}

// Device-side status words (one int each in a session's `status` buffer).
enum {
    ST_ERROR = 0,      // non-zero: a kernel gave up; bit values below
    ST_TICKET_BBOX,    // arrival counters of the last-block reductions
    ST_TICKET_SWING,
    ST_TICKET_NODE,
    ST_COUNT
};
enum {
    ERR_NAN = 1,       // swing/traction totals were not numbers
    ERR_WAIT = 2,      // a bounded wait on an mbarrier ran out
    ERR_BOUNDS = 4,    // a computed index or walk left its bounds (a bug)
};

// Speed-controller state on the device, in double (reference
// src/forceatlas2.c:445-485 runs it on the host; here it never leaves HBM).
struct SpeedState {
    double speed, efficiency;
    double total_swinging, total_traction;
    double jitter_tolerance;
    int n, pad;
};

// ---- precision traits -----------------------------------------------------
template <class R> struct RT;
template <> struct RT<float> {
    typedef float2 R2;
    typedef float4 R4;
};
template <> struct RT<double> {
    typedef double2 R2;
    typedef double4_32a R4;
};

// Traversal records of the n-1 regions of the Karras tree, in two arrays
// (a walk step reads 16 + 8 bytes in float, 32 + 8 in double):
//   rec_c[r] = (cx, cy, m, size^2);
//   rec_t[r] = (left, skip): the left child, and the next region that is not
//   a descendant (-1 at the end). A region of at most 8 nodes is never
//   opened; its left link carries its range of sorted nodes instead,
//   ~(first | (last - first) << 27), negative (first < 2^27).
__host__ __device__ __forceinline__ int bucket_pack(int first, int last)
{
    return ~(first | ((last - first) << 27));
}
__host__ __device__ __forceinline__ int bucket_first(int left) { return ~left & ((1 << 27) - 1); }
__host__ __device__ __forceinline__ int bucket_last(int left)
{
    return (~left & ((1 << 27) - 1)) + (~left >> 27);
}

// One CSR incidence: the node at the other end and the attraction strength.
template <class R> struct alignas(2 * sizeof(R) > 8 ? 16 : 8) Inc {
    int j;
    R coef;
};

// Per-region sums of the tree: bounding box, mass, sum m*x and sum m*y.
// Summed in plain float, sum m*x over a million nodes at coordinates ~1e4
// loses the centre of mass to ~1e-2 (the reference's float construction
// does). The FP64 path sums in double; the FP32 path in float-float (an
// unevaluated pair hi + lo kept exact by error-free transformations), which
// is as accurate for these sums and stays on the FP32 pipe (GB300's FP64
// rate is 1/64 of its FP32 rate).
struct ff2 {
    float hi, lo;
};
template <class R> struct Agg;
template <> struct alignas(32) Agg<double> {
    double minx, miny, maxx, maxy, m, mx, my, pad;
};
template <> struct alignas(16) Agg<float> {
    float minx, miny, maxx, maxy;
    ff2 m, mx, my, pad;
};

// Leaves of a device-side quadtree region list (fa2_gpu_repulse_bh):
// rr = (cx, cy, mass, size^2), ri = (start, count, last child, skip).
template <class R> struct QRegion {
    typename RT<R>::R4 rr;
    int4 ri;
};

inline int ceil_div(long long a, long long b) { return (int) ((a + b - 1) / b); }

} // namespace fa2cu

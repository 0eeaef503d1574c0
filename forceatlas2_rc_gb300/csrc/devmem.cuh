// devmem.cuh -- device buffers of a session, released together.
#pragma once

#include <cuda_runtime.h>
#include <vector>

namespace fa2cu {

struct DevMem {
    std::vector<void *> ptrs;
    double bytes = 0.0;
    bool failed = false;
    cudaError_t err = cudaSuccess;
    // With a pool: stream-ordered allocations on `s` from `pool` (no device
    // synchronisation on allocation or release). Dry: count bytes only.
    cudaMemPool_t pool = nullptr;
    cudaStream_t s = nullptr;
    bool dry = false;
    template <class T> T *get(size_t count)
    {
        if (failed) return nullptr;
        void *p = nullptr;
        const size_t b = (count > 0 ? count : 1) * sizeof(T);
        if (dry) {
            bytes += (double) b;
            return nullptr;
        }
        err = pool ? cudaMallocFromPoolAsync(&p, b, pool, s) : cudaMalloc(&p, b);
        if (err != cudaSuccess) {
            failed = true;
            return nullptr;
        }
        ptrs.push_back(p);
        bytes += (double) b;
        return (T *) p;
    }
    void release()
    {
        for (void *p : ptrs) {
            if (pool)
                cudaFreeAsync(p, s);
            else
                cudaFree(p);
        }
        ptrs.clear();
    }
};

} // namespace fa2cu

// dgx_pool.cpp -- device blocks of meshes and solvers, and the pool that
// recycles them.
//
// No counterpart in the reference, which allocates each array of its one solve
// with cudaMalloc at start-up (src/2d/main.cu).  Here a mesh or a solver is one
// allocation, and a request server, which creates and retires solves all the
// time, draws them from a BlockPool: free lists by size class, so a warm server
// neither allocates nor frees device memory (cudaFree waits for the whole
// device).  Blocks of up to kSlabBlock bytes are carved from 64 MiB slabs, so
// even a cold pool makes one cudaMalloc per slab; they stay in the pool until
// it is destroyed.  Larger blocks are allocated one by one and cached up to the
// pool's keep limit.
#include <cuda_runtime.h>

#include <vector>

#include "dgx_internal.h"

namespace dgx {

size_t BlockPool::size_class(size_t bytes) {
    if (bytes <= 4096) return 4096;
    if (bytes <= 65536) {
        size_t c = 4096;
        while (c < bytes) c <<= 1;
        return c;
    }
    const int e = 63 - __builtin_clzll(static_cast<unsigned long long>(bytes - 1));   // 2^e < bytes <= 2^(e+1)
    const size_t step = static_cast<size_t>(1) << (e - 3);
    return (bytes + step - 1) / step * step;
}

int BlockPool::get(size_t bytes, void **p, size_t *got) {
    const size_t cls = size_class(bytes);
    {
        std::lock_guard<std::mutex> lk(mu_);
        // the class itself or one of the next two (at most 25% larger)
        auto it = free_.lower_bound(cls);
        if (it != free_.end() && it->first <= cls + cls / 4) {
            *p = it->second;
            *got = it->first;
            if (it->first > kSlabBlock) cached_ -= it->first;
            free_.erase(it);
            ++hits_;
            return DGX_OK;
        }
        ++misses_;
        if (cls <= kSlabBlock) {
            if (slab_left_ < cls) {   // the rest of the current slab is left unused
                void *slab = nullptr;
                if (cudaMalloc(&slab, kSlabBytes) != cudaSuccess) {
                    cudaGetLastError();
                    *p = nullptr;
                    set_error("cudaMalloc of a %zu-byte slab failed", kSlabBytes);
                    return DGX_ERR_NOMEM;
                }
                slabs_.push_back(slab);
                slab_next_ = static_cast<char *>(slab);
                slab_left_ = kSlabBytes;
            }
            *p = slab_next_;
            *got = cls;
            slab_next_ += cls;
            slab_left_ -= cls;
            return DGX_OK;
        }
    }
    cudaError_t e = cudaMalloc(p, cls);
    if (e == cudaErrorMemoryAllocation) {
        cudaGetLastError();   // clear the allocation error, give the cache back and retry once
        trim();
        e = cudaMalloc(p, cls);
    }
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        set_error("cudaMalloc of %zu bytes failed: %s", cls, cudaGetErrorString(e));
        return DGX_ERR_NOMEM;
    }
    *got = cls;
    return DGX_OK;
}

void BlockPool::put(void *p, size_t bytes) {
    if (!p) return;
    {
        std::lock_guard<std::mutex> lk(mu_);
        if (bytes <= kSlabBlock) {   // carved from a slab: always kept
            free_.emplace(bytes, p);
            return;
        }
        if (cached_ + bytes <= keep_) {
            free_.emplace(bytes, p);
            cached_ += bytes;
            return;
        }
    }
    cudaFree(p);
}

void BlockPool::trim() {
    std::vector<void *> big;
    {
        std::lock_guard<std::mutex> lk(mu_);
        for (auto it = free_.begin(); it != free_.end();) {
            if (it->first > kSlabBlock) {
                big.push_back(it->second);
                it = free_.erase(it);
            } else {
                ++it;
            }
        }
        cached_ = 0;
    }
    for (void *p : big) cudaFree(p);
}

BlockPool::~BlockPool() {
    trim();
    for (void *s : slabs_) cudaFree(s);
}

size_t BlockPool::cached_bytes() {
    std::lock_guard<std::mutex> lk(mu_);
    return cached_;
}

int block_alloc(DeviceBlock &b, size_t bytes, BlockPool *pool) {
    b.pool = pool;
    if (pool) return pool->get(bytes, &b.base, &b.bytes);
    const cudaError_t e = cudaMalloc(&b.base, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        b.base = nullptr;
        set_error("cudaMalloc of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
        return DGX_ERR_NOMEM;
    }
    b.bytes = bytes;
    return DGX_OK;
}

void block_free(DeviceBlock &b) {
    if (!b.base) return;
    if (b.pool) b.pool->put(b.base, b.bytes);
    else cudaFree(b.base);
    b.base = nullptr;
    b.bytes = 0;
}

}  // namespace dgx

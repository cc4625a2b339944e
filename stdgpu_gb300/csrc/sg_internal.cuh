// Internal helpers shared by the library's translation units.
#ifndef SG_INTERNAL_CUH
#define SG_INTERNAL_CUH

#include <cuda_runtime.h>

#include <atomic>
#include <cstdint>

#include "stdgpu_gb300.h"

namespace sg
{
namespace detail
{

extern std::atomic<long long> g_launches;

// Switches a table just created (empty, nothing queued on it but its initialisation) to take keys until
// no slot is free, without the reference's excess-list accounting and without a synchronisation: the
// server's tables (unordered.cu).
void unordered_accounting_off(sg_unordered* table);

inline void
count_launch(long long n = 1)
{
    g_launches.fetch_add(n, std::memory_order_relaxed);
}

inline cudaStream_t
as_stream(void* s)
{
    return static_cast<cudaStream_t>(s);
}

// Device storage of every container goes through one allocator: cudaMalloc / cudaFree, or the pair a
// caller installs with sg_set_device_allocator (the reference's Allocator parameter,
// src/stdgpu/memory.h).  `live` counts allocations not yet freed, so the pair is only swapped while none
// made through the current one remain.
struct device_allocator
{
    std::atomic<sg_device_alloc_fn> alloc{ nullptr };
    std::atomic<sg_device_free_fn> release{ nullptr };
    std::atomic<void*> ctx{ nullptr };
    std::atomic<long long> live{ 0 };
};

inline device_allocator&
allocator()
{
    static device_allocator a;
    return a;
}

template <typename T>
inline cudaError_t
dev_malloc(T** p, size_t bytes)
{
    device_allocator& a = allocator();
    const sg_device_alloc_fn f = a.alloc.load();
    void* q = nullptr;
    if (f != nullptr)
    {
        q = f(bytes > 0 ? bytes : 1, a.ctx.load());
        if (q == nullptr)
        {
            *p = nullptr;
            return cudaErrorMemoryAllocation;
        }
    }
    else
    {
        const cudaError_t e = cudaMalloc(&q, bytes);
        if (e != cudaSuccess)
        {
            *p = nullptr;
            return e;
        }
    }
    a.live.fetch_add(1);
    *p = static_cast<T*>(q);
    return cudaSuccess;
}

inline void
dev_free(void* p)
{
    if (p == nullptr)
    {
        return;
    }
    device_allocator& a = allocator();
    const sg_device_free_fn f = a.release.load();
    if (f != nullptr)
    {
        // cudaFree waits for the device before it returns memory; a caller's release may hand the memory
        // to other users at once, so wait the same way
        cudaDeviceSynchronize();
        f(p, a.ctx.load());
    }
    else
    {
        cudaFree(p);
    }
    a.live.fetch_sub(1);
}

// One object's own allocator (sg_unordered_create_with_allocator); alloc == nullptr: the process-wide pair.
struct object_allocator
{
    sg_device_alloc_fn alloc = nullptr;
    sg_device_free_fn release = nullptr;
    void* ctx = nullptr;
};

template <typename T>
inline cudaError_t
obj_malloc(const object_allocator& oa, T** p, size_t bytes)
{
    if (oa.alloc == nullptr)
    {
        return dev_malloc(p, bytes);
    }
    void* q = oa.alloc(bytes > 0 ? bytes : 1, oa.ctx);
    *p = static_cast<T*>(q);
    return q == nullptr ? cudaErrorMemoryAllocation : cudaSuccess;
}

inline void
obj_free(const object_allocator& oa, void* p)
{
    if (p == nullptr)
    {
        return;
    }
    if (oa.alloc == nullptr)
    {
        dev_free(p);
        return;
    }
    cudaDeviceSynchronize(); // as cudaFree does, before the caller's release may hand the memory on
    oa.release(p, oa.ctx);
}

// Blocks per SM at which `kernel` is resident with `threads` threads, times the SM count.
template <typename Kernel>
int
persistent_grid(Kernel kernel, int threads, std::size_t smem = 0)
{
    int dev = 0;
    cudaGetDevice(&dev);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, threads, smem);
    if (per_sm < 1)
    {
        per_sm = 1;
    }
    return sms * per_sm;
}

inline int
grid_for(int64_t work_items, int items_per_block, int max_grid)
{
    int64_t g = (work_items + items_per_block - 1) / items_per_block;
    if (g < 1)
    {
        g = 1;
    }
    return static_cast<int>(g < max_grid ? g : max_grid);
}

} // namespace detail
} // namespace sg

#define SG_CUDA_TRY(expr)                                                                                              \
    do                                                                                                                 \
    {                                                                                                                  \
        cudaError_t sg_err_ = (expr);                                                                                  \
        if (sg_err_ != cudaSuccess)                                                                                    \
        {                                                                                                              \
            return sg_err_ == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA;                                   \
        }                                                                                                              \
    } while (0)

#define SG_LAUNCH_CHECK()                                                                                              \
    do                                                                                                                 \
    {                                                                                                                  \
        ::sg::detail::count_launch();                                                                                  \
        cudaError_t sg_err_ = cudaGetLastError();                                                                      \
        if (sg_err_ != cudaSuccess)                                                                                    \
        {                                                                                                              \
            return SG_ERR_CUDA;                                                                                        \
        }                                                                                                              \
    } while (0)

#endif

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

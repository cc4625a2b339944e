// Batched many-table entry points: thousands of independent unordered_set / unordered_map objects of
// uneven sizes built and probed in one launch per operation.
//
// All tables of a batch share one device arena (each table's probe groups contiguous, the layout and
// geometry of a single table: include/stdgpu_gb300/detail/layout.cuh) and a device array of per-table
// views.  An operation takes the keys of all tables concatenated, with per-table offsets in device
// memory.  A small kernel turns the offsets into a tile list -- tile x covers 32 consecutive keys of
// one table -- as a prefix count of tiles per table; a persistent kernel then walks the tiles
// (tile -> table by binary search of the prefix), running the same warp steps as the single-table
// kernels on that table's view.  No host work depends on the sizes, so a sequence of batched calls
// can be captured in a CUDA graph and replayed.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <new>
#include <vector>

#include "sg_internal.cuh"
#include "stdgpu_gb300.h"
#include "table_core.cuh"

namespace sg
{
namespace detail
{

constexpr int kInitChunkUnits = 1 << 14; // 16-byte units per init work item (256 KiB)

struct init_chunk
{
    int32_t table;
    int32_t pad;
    int64_t unit_begin; // 16-byte units within the table
    int64_t unit_end;
};

// Prefix of tile counts: prefix[t] = sum over u < t of ceil(n_u / 32); prefix[n] = all tiles.
__global__ void __launch_bounds__(1024)
k_batch_tiles(const int64_t* offsets, int32_t n, int64_t* prefix, bool has_keys)
{
    __shared__ long long part[1024];
    const int64_t per = (static_cast<int64_t>(n) + blockDim.x - 1) / blockDim.x;
    const int64_t lo = threadIdx.x * per;
    const int64_t hi = lo + per < n ? lo + per : n;
    long long s = 0;
    for (int64_t t = lo; t < hi; ++t)
    {
        const int64_t cnt = has_keys ? offsets[t + 1] - offsets[t] : 0;
        s += cnt > 0 ? (cnt + 31) / 32 : 0;
    }
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        long long run = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x); ++w)
        {
            const long long x = part[w];
            part[w] = run;
            run += x;
        }
        prefix[n] = run;
    }
    __syncthreads();
    long long run = part[threadIdx.x];
    for (int64_t t = lo; t < hi; ++t)
    {
        prefix[t] = run;
        const int64_t cnt = has_keys ? offsets[t + 1] - offsets[t] : 0;
        run += cnt > 0 ? (cnt + 31) / 32 : 0;
    }
}

// Table of tile x: the last t with prefix[t] <= x (binary search by lane 0, broadcast to the warp).
SG_D int32_t
tile_table(const int64_t* prefix, int32_t n, int64_t x)
{
    int32_t t = 0;
    if ((threadIdx.x & 31) == 0)
    {
        int32_t lo = 0, hi = n; // invariant: prefix[lo] <= x < prefix[hi]
        while (hi - lo > 1)
        {
            const int32_t mid = (lo + hi) >> 1;
            if (__ldg(prefix + mid) <= x)
            {
                lo = mid;
            }
            else
            {
                hi = mid;
            }
        }
        t = lo;
    }
    return __shfl_sync(0xffffffffu, t, 0);
}

SG_D unsigned long long
warp_sum(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    return v;
}

enum batch_op : int
{
    kOpInsertAos = 0,
    kOpInsertSoa = 1,
    kOpErase = 2,
    kOpFind = 3,
    kOpContains = 4
};

// Persistent walk over the tile list; each warp takes `tiles_per_step` consecutive tiles at a time.
template <int KIND, int OP, int THREADS>
__global__ void __launch_bounds__(THREADS)
k_batch(const dview* views, const int64_t* offsets, const int64_t* prefix, int32_t n, int tiles_per_step,
        const void* in0, const void* in1, void* out_vals, uint8_t* out_flags)
{
    const tile_lanes L;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int64_t tiles = __ldg(prefix + n);
    unsigned long long retry = 0;
    for (int64_t x0 = warp * tiles_per_step; x0 < tiles; x0 += nwarps * tiles_per_step)
    {
        const int64_t x1 = x0 + tiles_per_step < tiles ? x0 + tiles_per_step : tiles;
        for (int64_t x = x0; x < x1; ++x)
        {
            const int32_t tb = tile_table(prefix, n, x);
            const dview t = views[tb];
            const int64_t end = __ldg(offsets + tb + 1);
            const int64_t i = __ldg(offsets + tb) + (x - __ldg(prefix + tb)) * 32 + L.lane;
            const bool valid = i < end;
            step_counts c;
            if constexpr (OP == kOpInsertAos || OP == kOpInsertSoa)
            {
                insert_step<KIND, OP == kOpInsertAos>(t, L, in0, in1, i, valid, out_flags, c);
                const unsigned long long d = warp_sum(c.done), r = warp_sum(c.refused), u = warp_sum(c.reused);
                retry += c.retry;
                if (L.lane == 0)
                {
                    if (d != 0)
                    {
                        atomicAdd(&t.hdr->size, d);
                    }
                    if (r != 0)
                    {
                        atomicAdd(&t.hdr->refused, r);
                    }
                    if (u != 0)
                    {
                        atomicAdd(&t.hdr->tombstones, 0ull - u);
                    }
                }
            }
            else if constexpr (OP == kOpErase)
            {
                erase_step<KIND>(t, L, in0, i, valid, out_flags, c);
                const unsigned long long d = warp_sum(c.done), o = warp_sum(c.oob);
                if (L.lane == 0 && d != 0)
                {
                    atomicAdd(&t.hdr->size, 0ull - d);
                    atomicAdd(&t.hdr->tombstones, d - o);
                }
            }
            else
            {
                find_step<KIND, OP == kOpFind>(t, L, in0, i, valid, out_vals, out_flags);
            }
        }
    }
    if (retry != 0)
    {
        atomicOr(&views[0].hdr->error, kErrRetry);
    }
}

// Init of all tables: work items of up to kInitChunkUnits 16-byte units of one table.
template <int KIND>
__global__ void __launch_bounds__(256)
k_batch_init(const dview* views, const init_chunk* chunks, int64_t nchunks)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    constexpr int G = C::slots_per_group;
    for (int64_t c = blockIdx.x; c < nchunks; c += gridDim.x)
    {
        const init_chunk ch = chunks[c];
        const dview t = views[ch.table];
        uint4* base = reinterpret_cast<uint4*>(t.slots);
        for (int64_t u = ch.unit_begin + threadIdx.x; u < ch.unit_end; u += blockDim.x)
        {
            const int64_t first = u * C::slots_per_lane;
            if (first + C::slots_per_lane <= t.total || first >= static_cast<int64_t>(t.num_groups) * G)
            {
                base[u] = make_uint4(~0u, ~0u, ~0u, ~0u);
            }
            else
            {
                uint4 d = make_uint4(~0u, ~0u, ~0u, ~0u);
                char* bytes = reinterpret_cast<char*>(&d);
                for (int s = 0; s < C::slots_per_lane; ++s)
                {
                    if (first + s >= t.total)
                    {
                        *reinterpret_cast<K*>(bytes + s * C::slot_bytes) = C::tomb_key;
                    }
                }
                base[u] = d;
            }
        }
        if (ch.unit_begin == 0 && threadIdx.x == 0)
        {
            t.hdr->size = 0;
            t.hdr->refused = 0;
            t.hdr->tombstones = 0;
            t.hdr->special_state[0] = 0;
            t.hdr->special_state[1] = 0;
            t.hdr->error = 0;
            t.hdr->count = 0;
        }
    }
}

__global__ void
k_batch_gather_sizes(const dview* views, int32_t n, long long* sizes)
{
    for (int32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    {
        sizes[t] = static_cast<long long>(views[t].hdr->size);
    }
}

} // namespace detail
} // namespace sg

using namespace sg::detail;

struct sg_table_batch
{
    int32_t kind;
    int32_t n;
    int32_t threads;       // launch shape of the walking kernels (autotuned)
    int32_t blocks_per_sm;
    int32_t tiles_per_step;
    int32_t sms;
    char* arena;
    table_header* headers;
    dview* views;            // device
    std::vector<dview> host_views;
    std::vector<int64_t> capacities, bucket_counts, totals;
    init_chunk* chunks;      // device
    int64_t nchunks;
    int64_t* prefix;         // device, n + 1
    long long* sizes_dev;    // device, n
    long long* sizes_host;   // pinned, n
    int64_t arena_bytes;
    unsigned int* locks;     // stripe locks of native device inserts, shared by the batch's tables
};

constexpr int64_t kBatchInsertLocks = int64_t{ 1 } << 16;

namespace
{

inline void
batch_geometry(int64_t capacity, int kind, int64_t* bucket_count, int64_t* total, int64_t* groups, int* bits)
{
    int64_t b = 0, e = 0;
    reference_geometry(capacity, &b, &e);
    const int spg = kGroupBytes / slot_bytes_of_kind(kind);
    *bucket_count = b;
    *total = b + e;
    *groups = (*total + spg - 1) / spg;
    *bits = log2_exact(b);
}

template <int KIND>
struct batch_launch
{
    template <int OP, int THREADS>
    static sg_status
    go(sg_table_batch* b, const int64_t* offsets, const void* in0, const void* in1, void* out_vals,
       uint8_t* out_flags, cudaStream_t s)
    {
        int per_sm = 0;
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<KIND, OP, THREADS>, THREADS, 0);
        per_sm = per_sm < 1 ? 1 : per_sm;
        const int want = b->blocks_per_sm > 0 ? (b->blocks_per_sm < per_sm ? b->blocks_per_sm : per_sm) : per_sm;
        k_batch<KIND, OP, THREADS><<<b->sms * want, THREADS, 0, s>>>(b->views, offsets, b->prefix, b->n,
                                                                      b->tiles_per_step, in0, in1, out_vals,
                                                                      out_flags);
        SG_LAUNCH_CHECK();
        return SG_OK;
    }

    template <int OP>
    static sg_status
    run_op(sg_table_batch* b, const int64_t* offsets, const void* in0, const void* in1, void* out_vals,
           uint8_t* out_flags, cudaStream_t s)
    {
        switch (b->threads)
        {
            case 128:
                return go<OP, 128>(b, offsets, in0, in1, out_vals, out_flags, s);
            case 512:
                return go<OP, 512>(b, offsets, in0, in1, out_vals, out_flags, s);
            default:
                return go<OP, 256>(b, offsets, in0, in1, out_vals, out_flags, s);
        }
    }

    static sg_status
    run(sg_table_batch* b, int op, const int64_t* offsets, const void* in0, const void* in1, void* out_vals,
        uint8_t* out_flags, cudaStream_t s)
    {
        switch (op)
        {
            case kOpInsertAos:
                return run_op<kOpInsertAos>(b, offsets, in0, in1, out_vals, out_flags, s);
            case kOpInsertSoa:
                return run_op<kOpInsertSoa>(b, offsets, in0, in1, out_vals, out_flags, s);
            case kOpErase:
                return run_op<kOpErase>(b, offsets, in0, in1, out_vals, out_flags, s);
            case kOpFind:
                return run_op<kOpFind>(b, offsets, in0, in1, out_vals, out_flags, s);
            default:
                return run_op<kOpContains>(b, offsets, in0, in1, out_vals, out_flags, s);
        }
    }

    static sg_status
    init(sg_table_batch* b, cudaStream_t s)
    {
        const int grid = b->sms * 8;
        k_batch_init<KIND><<<grid, 256, 0, s>>>(b->views, b->chunks, b->nchunks);
        SG_LAUNCH_CHECK();
        return SG_OK;
    }
};

sg_status
dispatch_op(sg_table_batch* b, int op, const int64_t* offsets, const void* in0, const void* in1, void* out_vals,
            uint8_t* out_flags, cudaStream_t s)
{
    // a NULL key array (all ranges empty, as an empty tensor gives) walks no tile
    k_batch_tiles<<<1, 1024, 0, s>>>(offsets, b->n, b->prefix, in0 != nullptr);
    SG_LAUNCH_CHECK();
    switch (b->kind)
    {
        case 0:
            return batch_launch<0>::run(b, op, offsets, in0, in1, out_vals, out_flags, s);
        case 1:
            return batch_launch<1>::run(b, op, offsets, in0, in1, out_vals, out_flags, s);
        case 2:
            return batch_launch<2>::run(b, op, offsets, in0, in1, out_vals, out_flags, s);
        case 3:
            return batch_launch<3>::run(b, op, offsets, in0, in1, out_vals, out_flags, s);
        case 4:
            return batch_launch<4>::run(b, op, offsets, in0, in1, out_vals, out_flags, s);
        case 5:
            return batch_launch<5>::run(b, op, offsets, in0, in1, out_vals, out_flags, s);
        default:
            return SG_ERR_BAD_ARG;
    }
}

sg_status
dispatch_init(sg_table_batch* b, cudaStream_t s)
{
    switch (b->kind)
    {
        case 0:
            return batch_launch<0>::init(b, s);
        case 1:
            return batch_launch<1>::init(b, s);
        case 2:
            return batch_launch<2>::init(b, s);
        case 3:
            return batch_launch<3>::init(b, s);
        case 4:
            return batch_launch<4>::init(b, s);
        case 5:
            return batch_launch<5>::init(b, s);
        default:
            return SG_ERR_BAD_ARG;
    }
}

bool
args_ok(const sg_table_batch* b, const void* in0, const int64_t* offsets)
{
    (void)in0; // NULL keys are allowed: the call then walks no tile
    return b != nullptr && offsets != nullptr;
}

} // namespace

extern "C" {

sg_status
sg_batch_create(int32_t kind, int32_t n_tables, const int64_t* capacities, void* stream, sg_table_batch** out)
{
    if (out == nullptr || capacities == nullptr || n_tables <= 0 || kind < SG_SET_U32 || kind > SG_MAP_U32_U64)
    {
        return SG_ERR_BAD_ARG;
    }
    *out = nullptr;
    auto* b = new (std::nothrow) sg_table_batch{};
    if (b == nullptr)
    {
        return SG_ERR_OOM;
    }
    b->kind = kind;
    b->n = n_tables;
    b->threads = 256;
    b->blocks_per_sm = 0;
    b->tiles_per_step = 1;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, dev);
    b->capacities.assign(capacities, capacities + n_tables);
    std::vector<int64_t> group_offset(n_tables + 1, 0);
    std::vector<int> bits(n_tables);
    std::vector<int64_t> groups(n_tables);
    b->bucket_counts.resize(n_tables);
    b->totals.resize(n_tables);
    for (int32_t t = 0; t < n_tables; ++t)
    {
        if (capacities[t] <= 0)
        {
            delete b;
            return SG_ERR_BAD_ARG;
        }
        batch_geometry(capacities[t], kind, &b->bucket_counts[t], &b->totals[t], &groups[t], &bits[t]);
        if (b->totals[t] >= (int64_t{ 1 } << 31))
        {
            delete b;
            return SG_ERR_BAD_ARG;
        }
        group_offset[t + 1] = group_offset[t] + groups[t] + 1; // + tail group of out-of-band keys
    }
    b->arena_bytes = group_offset[n_tables] * kGroupBytes;
    std::vector<init_chunk> chunks;
    for (int32_t t = 0; t < n_tables; ++t)
    {
        const int64_t units = (groups[t] + 1) * (kGroupBytes / 16);
        for (int64_t u = 0; u < units; u += kInitChunkUnits)
        {
            chunks.push_back(init_chunk{ t, 0, u, u + kInitChunkUnits < units ? u + kInitChunkUnits : units });
        }
    }
    b->nchunks = static_cast<int64_t>(chunks.size());
    cudaError_t e = sg::detail::dev_malloc(&b->arena, static_cast<size_t>(b->arena_bytes));
    if (e == cudaSuccess)
    {
        e = sg::detail::dev_malloc(&b->headers, sizeof(table_header) * n_tables);
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::dev_malloc(&b->views, sizeof(dview) * n_tables);
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::dev_malloc(&b->chunks, sizeof(init_chunk) * chunks.size());
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::dev_malloc(&b->prefix, sizeof(int64_t) * (n_tables + 1));
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::dev_malloc(&b->sizes_dev, sizeof(long long) * n_tables);
    }
    if (e == cudaSuccess)
    {
        e = cudaMallocHost(&b->sizes_host, sizeof(long long) * n_tables);
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::dev_malloc(&b->locks, sizeof(unsigned int) * kBatchInsertLocks);
    }
    if (e == cudaSuccess)
    {
        e = cudaMemsetAsync(b->locks, 0, sizeof(unsigned int) * kBatchInsertLocks, as_stream(stream));
    }
    if (e != cudaSuccess)
    {
        sg_batch_destroy(b);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA;
    }
    b->host_views.resize(n_tables);
    for (int32_t t = 0; t < n_tables; ++t)
    {
        b->host_views[t] = dview{ b->arena + group_offset[t] * kGroupBytes, b->headers + t,
                                  static_cast<uint32_t>(groups[t]), static_cast<uint32_t>(b->totals[t]), bits[t] };
    }
    cudaStream_t s = as_stream(stream);
    e = cudaMemcpyAsync(b->views, b->host_views.data(), sizeof(dview) * n_tables, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess)
    {
        e = cudaMemcpyAsync(b->chunks, chunks.data(), sizeof(init_chunk) * chunks.size(), cudaMemcpyHostToDevice, s);
    }
    if (e == cudaSuccess)
    {
        e = cudaStreamSynchronize(s); // host vectors above are released on return
    }
    if (e != cudaSuccess)
    {
        sg_batch_destroy(b);
        return SG_ERR_CUDA;
    }
    const sg_status st = dispatch_init(b, s);
    if (st != SG_OK)
    {
        sg_batch_destroy(b);
        return st;
    }
    *out = b;
    return SG_OK;
}

sg_status
sg_batch_destroy(sg_table_batch* b)
{
    if (b == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaDeviceSynchronize();
    sg::detail::dev_free(b->arena);
    sg::detail::dev_free(b->headers);
    sg::detail::dev_free(b->views);
    sg::detail::dev_free(b->chunks);
    sg::detail::dev_free(b->prefix);
    sg::detail::dev_free(b->sizes_dev);
    sg::detail::dev_free(b->locks);
    if (b->sizes_host != nullptr)
    {
        cudaFreeHost(b->sizes_host);
    }
    delete b;
    return SG_OK;
}

sg_status
sg_batch_configure(sg_table_batch* b, int32_t threads_per_block, int32_t blocks_per_sm, int32_t tiles_per_step)
{
    if (b == nullptr || (threads_per_block != 128 && threads_per_block != 256 && threads_per_block != 512) ||
        blocks_per_sm < 0 || tiles_per_step < 1 || tiles_per_step > 64)
    {
        return SG_ERR_BAD_ARG;
    }
    b->threads = threads_per_block;
    b->blocks_per_sm = blocks_per_sm;
    b->tiles_per_step = tiles_per_step;
    return SG_OK;
}

sg_status
sg_batch_clear(sg_table_batch* b, void* stream)
{
    if (b == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    return dispatch_init(b, as_stream(stream));
}

sg_status
sg_batch_insert(sg_table_batch* b, const void* values, const int64_t* offsets, uint8_t* out_inserted, void* stream)
{
    if (!args_ok(b, values, offsets))
    {
        return SG_ERR_BAD_ARG;
    }
    return dispatch_op(b, kOpInsertAos, offsets, values, nullptr, nullptr, out_inserted, as_stream(stream));
}

sg_status
sg_batch_insert_kv(sg_table_batch* b, const void* keys, const void* mapped, const int64_t* offsets,
                   uint8_t* out_inserted, void* stream)
{
    if (!args_ok(b, keys, offsets))
    {
        return SG_ERR_BAD_ARG;
    }
    return dispatch_op(b, kOpInsertSoa, offsets, keys, mapped, nullptr, out_inserted, as_stream(stream));
}

sg_status
sg_batch_erase(sg_table_batch* b, const void* keys, const int64_t* offsets, uint8_t* out_erased, void* stream)
{
    if (!args_ok(b, keys, offsets))
    {
        return SG_ERR_BAD_ARG;
    }
    return dispatch_op(b, kOpErase, offsets, keys, nullptr, nullptr, out_erased, as_stream(stream));
}

sg_status
sg_batch_find(sg_table_batch* b, const void* keys, const int64_t* offsets, void* out_mapped, uint8_t* out_found,
              void* stream)
{
    if (!args_ok(b, keys, offsets))
    {
        return SG_ERR_BAD_ARG;
    }
    const bool is_map = b->kind >= SG_MAP_U64_U32;
    return dispatch_op(b, kOpFind, offsets, keys, nullptr, is_map ? out_mapped : nullptr, out_found,
                       as_stream(stream));
}

sg_status
sg_batch_contains(sg_table_batch* b, const void* keys, const int64_t* offsets, uint8_t* out_flags, void* stream)
{
    if (!args_ok(b, keys, offsets) || (keys != nullptr && out_flags == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    return dispatch_op(b, kOpContains, offsets, keys, nullptr, nullptr, out_flags, as_stream(stream));
}

sg_status
sg_batch_sizes(sg_table_batch* b, void* stream, int64_t* out_sizes)
{
    if (b == nullptr || out_sizes == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = as_stream(stream);
    k_batch_gather_sizes<<<(b->n + 255) / 256, 256, 0, s>>>(b->views, b->n, b->sizes_dev);
    SG_LAUNCH_CHECK();
    SG_CUDA_TRY(cudaMemcpyAsync(b->sizes_host, b->sizes_dev, sizeof(long long) * b->n, cudaMemcpyDeviceToHost, s));
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    for (int32_t t = 0; t < b->n; ++t)
    {
        out_sizes[t] = static_cast<int64_t>(b->sizes_host[t]);
    }
    return SG_OK;
}

sg_status
sg_batch_view_of(const sg_table_batch* b, int32_t table, sg_unordered_view* out)
{
    if (b == nullptr || out == nullptr || table < 0 || table >= b->n)
    {
        return SG_ERR_BAD_ARG;
    }
    const dview& v = b->host_views[table];
    out->slots = v.slots;
    out->header = v.hdr;
    out->num_groups = v.num_groups;
    out->total_count = v.total;
    out->bucket_count = b->bucket_counts[table];
    out->bucket_bits = v.bits;
    out->kind = b->kind;
    out->insert_locks = b->locks;
    out->lock_mask = kBatchInsertLocks - 1;
    return SG_OK;
}

sg_status
sg_batch_info(const sg_table_batch* b, int64_t* out_storage_bytes, int32_t* out_n_tables)
{
    if (b == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    if (out_storage_bytes != nullptr)
    {
        *out_storage_bytes = b->arena_bytes;
    }
    if (out_n_tables != nullptr)
    {
        *out_n_tables = b->n;
    }
    return SG_OK;
}

} // extern "C"

// The plain one-call-per-table paths, driven from native code: the comparators that the batched and the
// served modes are measured against.  Each is the loop a C++ user of the library writes -- one C-ABI call
// per table and operation (and, for the request stream, a stream synchronisation after each request) --
// so the comparison carries no interpreter overhead.  No counterpart in the reference, whose users make
// these calls through its C++ template API.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdint>
#include <unordered_map>
#include <vector>

#include "stdgpu_gb300.h"

#if defined(__GNUC__)
#define SGC_API extern "C" __attribute__((visibility("default")))
#else
#define SGC_API extern "C"
#endif

namespace
{

using clock_type = std::chrono::steady_clock;

const char*
at(const void* base, int64_t elem, int64_t bytes)
{
    return static_cast<const char*>(base) + elem * bytes;
}

// The server's growth policy on a plain table, before an insert of n keys: bound is an upper bound of the
// table's size (exact after a read, plus the keys inserted since).
sg_status
grow_before_insert(sg_unordered* h, int32_t kind, int64_t n, void* stream, int64_t& bound, int64_t& grown)
{
    sg_geometry g{};
    sg_status st = sg_unordered_geometry(h, &g);
    if (st != SG_OK)
    {
        return st;
    }
    if (bound + n > g.max_size * 85 / 100)
    {
        st = sg_unordered_size(h, stream, &bound);
        if (st != SG_OK)
        {
            return st;
        }
        if (bound + n > g.max_size * 85 / 100)
        {
            int64_t cap = g.capacity;
            sg_geometry ng{};
            do
            {
                cap *= 2;
                st = sg_unordered_geometry_for(kind, cap, &ng);
                if (st != SG_OK)
                {
                    return st;
                }
            } while (bound + n > ng.max_size * 85 / 100);
            st = sg_unordered_rehash(h, cap, stream);
            if (st != SG_OK)
            {
                return st;
            }
            ++grown;
        }
    }
    bound += n;
    return SG_OK;
}

} // namespace

// Many small tables: `steps` times, for every table t, sg_unordered_clear, sg_unordered_insert_kv of its keys
// [offsets[t], offsets[t+1]) and sg_unordered_contains of the same number of queries into out_flags, all on
// one stream without synchronisation between calls.  gpu_ms: CUDA-event time per step; host_ms: wall time
// per step including the final synchronisation.
SGC_API sg_status
sgc_plain_tables_steps(sg_unordered* const* tables, int64_t n_tables, const void* keys, const void* queries,
                       const int64_t* offsets, int32_t key_bytes, uint8_t* out_flags, int32_t steps, void* stream,
                       double* gpu_ms, double* host_ms)
{
    if (tables == nullptr || offsets == nullptr || steps < 1 || (key_bytes != 4 && key_bytes != 8))
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    cudaEvent_t a = nullptr, b = nullptr;
    if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess)
    {
        return SG_ERR_CUDA;
    }
    if (cudaStreamSynchronize(s) != cudaSuccess)
    {
        return SG_ERR_CUDA;
    }
    const auto t0 = clock_type::now();
    cudaEventRecord(a, s);
    sg_status st = SG_OK;
    for (int32_t k = 0; k < steps && st == SG_OK; ++k)
    {
        for (int64_t t = 0; t < n_tables && st == SG_OK; ++t)
        {
            const int64_t lo = offsets[t];
            const int64_t n = offsets[t + 1] - lo;
            st = sg_unordered_clear(tables[t], stream);
            if (st == SG_OK)
            {
                st = sg_unordered_insert_kv(tables[t], at(keys, lo, key_bytes), nullptr, n, nullptr, stream);
            }
            if (st == SG_OK)
            {
                st = sg_unordered_contains(tables[t], at(queries, lo, key_bytes), n, out_flags + lo, stream);
            }
        }
    }
    cudaEventRecord(b, s);
    const bool synced = cudaEventSynchronize(b) == cudaSuccess;
    const auto t1 = clock_type::now();
    float ms = 0.0F;
    cudaEventElapsedTime(&ms, a, b);
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (st != SG_OK)
    {
        return st;
    }
    if (!synced)
    {
        return SG_ERR_CUDA;
    }
    if (gpu_ms != nullptr)
    {
        *gpu_ms = static_cast<double>(ms) / steps;
    }
    if (host_ms != nullptr)
    {
        *host_ms = std::chrono::duration<double, std::milli>(t1 - t0).count() / steps;
    }
    return SG_OK;
}

// A request stream on plain tables, one request at a time in submission order: the request's call on its
// table (insert_kv / find / erase, sg_request's fields as for the server) on one stream.
//   sync_each != 0: the serial plain path -- after each call the stream is synchronised; request i is not
//                   issued before arrivals_s[i] seconds after the start (nullable: all at once), and
//                   latencies_us[i] is its completion minus its arrival (or its issue, without arrivals).
//   sync_each == 0: back to back without synchronisation (the device time of the stream's kernels).
// kernel_us (nullable): each request's device time from CUDA events around its call.  wall_s: wall time of
// the whole stream.
//   grow_kind >= 0 (the tables' kind): before an insert that could take its table past 85 % of max_size(),
//                   the table's size is read and, where needed, the table is rehashed (sg_unordered_rehash)
//                   to the first doubling of its capacity that holds the insert -- the growth policy of the
//                   server, as a plain caller applies it; *rehashes counts them (nullable).
SGC_API sg_status
sgc_serial_replay(sg_unordered* const* tables, const sg_request* reqs, int64_t n, const double* arrivals_s,
                  int32_t sync_each, void* stream, double* latencies_us, float* kernel_us, double* wall_s,
                  int32_t grow_kind, int64_t* rehashes)
{
    if (tables == nullptr || (n > 0 && reqs == nullptr) || n < 0)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    std::vector<cudaEvent_t> ev;
    if (kernel_us != nullptr)
    {
        ev.resize(static_cast<size_t>(2 * n), nullptr);
        for (auto& e : ev)
        {
            if (cudaEventCreate(&e) != cudaSuccess)
            {
                for (auto& x : ev)
                {
                    if (x != nullptr)
                    {
                        cudaEventDestroy(x);
                    }
                }
                return SG_ERR_CUDA;
            }
        }
    }
    if (cudaStreamSynchronize(s) != cudaSuccess)
    {
        return SG_ERR_CUDA;
    }
    sg_status st = SG_OK;
    std::unordered_map<int32_t, int64_t> size_bound; // per table: exact after a read, plus keys inserted since
    int64_t grown = 0;
    const auto t0 = clock_type::now();
    for (int64_t i = 0; i < n && st == SG_OK; ++i)
    {
        const sg_request& r = reqs[i];
        auto due = t0;
        if (arrivals_s != nullptr)
        {
            due = t0 + std::chrono::duration_cast<clock_type::duration>(std::chrono::duration<double>(arrivals_s[i]));
            while (clock_type::now() < due)
            {
            }
        }
        const auto issued = clock_type::now();
        if (!ev.empty())
        {
            cudaEventRecord(ev[2 * i], s);
        }
        sg_unordered* h = tables[r.table];
        if (r.op == SG_SERVER_INSERT && grow_kind >= 0)
        {
            st = grow_before_insert(h, grow_kind, r.n, stream, size_bound[r.table], grown);
        }
        if (st != SG_OK)
        {
            break;
        }
        if (r.op == SG_SERVER_INSERT)
        {
            st = sg_unordered_insert_kv(h, r.keys, r.mapped, r.n, r.out_flags, stream);
        }
        else if (r.op == SG_SERVER_FIND)
        {
            st = sg_unordered_find(h, r.keys, r.n, r.out_mapped, r.out_flags, stream);
        }
        else if (r.op == SG_SERVER_ERASE)
        {
            st = sg_unordered_erase(h, r.keys, r.n, r.out_flags, stream);
        }
        else
        {
            st = SG_ERR_BAD_ARG;
        }
        if (!ev.empty())
        {
            cudaEventRecord(ev[2 * i + 1], s);
        }
        if (sync_each != 0)
        {
            if (cudaStreamSynchronize(s) != cudaSuccess)
            {
                st = SG_ERR_CUDA;
            }
            if (latencies_us != nullptr)
            {
                const auto from = arrivals_s != nullptr ? due : issued;
                latencies_us[i] = std::chrono::duration<double, std::micro>(clock_type::now() - from).count();
            }
        }
    }
    if (cudaStreamSynchronize(s) != cudaSuccess && st == SG_OK)
    {
        st = SG_ERR_CUDA;
    }
    const auto t1 = clock_type::now();
    if (wall_s != nullptr)
    {
        *wall_s = std::chrono::duration<double>(t1 - t0).count();
    }
    if (rehashes != nullptr)
    {
        *rehashes = grown;
    }
    for (int64_t i = 0; i < static_cast<int64_t>(ev.size()) / 2; ++i)
    {
        float ms = 0.0F;
        cudaEventElapsedTime(&ms, ev[2 * i], ev[2 * i + 1]);
        kernel_us[i] = ms * 1000.0F;
    }
    for (auto& e : ev)
    {
        cudaEventDestroy(e);
    }
    return st;
}

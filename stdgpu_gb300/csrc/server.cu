// Served request stream over device-resident tables (no counterpart in the reference).
//
// A scheduler thread keeps tables resident in HBM and turns submitted insert / find / erase requests
// into launches.  Continuous batching: whenever a launch slot is free, every table that has pending
// requests and nothing in flight contributes its longest run of consecutive same-operation requests;
// all runs of one operation go into one segmented launch (one segment per request), the launches of a
// wave go to different streams, and requests that arrive while earlier waves are on the GPU join the
// next wave.  A table stays busy until its wave completes, so every table sees its requests in
// submission order.  Tables are admitted, and grown before an insert run that would pass 85 % of
// max_size(), only while the HBM budget allows; otherwise the request is refused (SG_ERR_BUDGET)
// rather than spilled.  Latency is measured per request from submission to completion.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <unordered_map>
#include <vector>

#include "sg_internal.cuh"
#include "stdgpu_gb300.h"
#include "table_core.cuh"

namespace sg
{
namespace detail
{

// One request's share of a segmented launch.
struct seg_desc
{
    dview view;
    const void* in0;
    const void* in1;
    void* out_vals;
    uint8_t* out_flags;
    int64_t n;
};

constexpr int kSegThreads = 128;

SG_D int32_t
segment_of(const int64_t* prefix, int32_t nseg, int64_t x)
{
    int32_t t = 0;
    if ((threadIdx.x & 31) == 0)
    {
        int32_t lo = 0, hi = nseg; // prefix[lo] <= x < prefix[hi]
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
seg_warp_sum(unsigned long long v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        v += __shfl_xor_sync(0xffffffffu, v, o);
    }
    return v;
}

// OP: 0 insert (key / mapped arrays), 1 find, 2 erase.  prefix[s] = tiles before segment s.  Each warp
// walks kSegTilesPerStep consecutive tiles at a time, looks the segment up again only when it crosses
// a segment boundary, and adds its counts to the segment's table when it leaves the segment.
constexpr int kSegTilesPerStep = 8;

template <int KIND, int OP>
__global__ void __launch_bounds__(kSegThreads)
k_segments(const seg_desc* segs, const int64_t* prefix, int32_t nseg)
{
    const tile_lanes L;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const int64_t tiles = __ldg(prefix + nseg);
    for (int64_t x0 = warp * kSegTilesPerStep; x0 < tiles; x0 += nwarps * kSegTilesPerStep)
    {
        const int64_t x1 = x0 + kSegTilesPerStep < tiles ? x0 + kSegTilesPerStep : tiles;
        int32_t s = segment_of(prefix, nseg, x0);
        seg_desc d = segs[s];
        int64_t s_begin = __ldg(prefix + s);
        int64_t s_end = __ldg(prefix + s + 1);
        step_counts c;
        for (int64_t x = x0; x < x1; ++x)
        {
            if (x >= s_end)
            {
                // leaving segment s: flush its counts, move to the next non-empty segment
                if constexpr (OP != 1)
                {
                    const unsigned long long dn = seg_warp_sum(c.done), rf = seg_warp_sum(c.refused),
                                             ru = seg_warp_sum(c.reused), ob = seg_warp_sum(c.oob);
                    if (L.lane == 0 && (dn | rf | ru) != 0)
                    {
                        if (OP == 0)
                        {
                            atomicAdd(&d.view.hdr->size, dn);
                            atomicAdd(&d.view.hdr->refused, rf);
                            atomicAdd(&d.view.hdr->tombstones, 0ull - ru);
                        }
                        else
                        {
                            atomicAdd(&d.view.hdr->size, 0ull - dn);
                            atomicAdd(&d.view.hdr->tombstones, dn - ob);
                        }
                    }
                    c = step_counts{};
                }
                s = segment_of(prefix, nseg, x);
                d = segs[s];
                s_begin = __ldg(prefix + s);
                s_end = __ldg(prefix + s + 1);
            }
            const int64_t i = (x - s_begin) * 32 + L.lane;
            const bool valid = i < d.n;
            if constexpr (OP == 0)
            {
                insert_step<KIND, false>(d.view, L, d.in0, d.in1, i, valid, d.out_flags, c);
            }
            else if constexpr (OP == 1)
            {
                find_step<KIND, true>(d.view, L, d.in0, i, valid, d.out_vals, d.out_flags);
            }
            else
            {
                erase_step<KIND>(d.view, L, d.in0, i, valid, d.out_flags, c);
            }
        }
        if constexpr (OP != 1)
        {
            const unsigned long long dn = seg_warp_sum(c.done), rf = seg_warp_sum(c.refused),
                                     ru = seg_warp_sum(c.reused), ob = seg_warp_sum(c.oob);
            if (L.lane == 0 && (dn | rf | ru) != 0)
            {
                if (OP == 0)
                {
                    atomicAdd(&d.view.hdr->size, dn);
                    atomicAdd(&d.view.hdr->refused, rf);
                    atomicAdd(&d.view.hdr->tombstones, 0ull - ru);
                }
                else
                {
                    atomicAdd(&d.view.hdr->size, 0ull - dn);
                    atomicAdd(&d.view.hdr->tombstones, dn - ob);
                }
            }
        }
    }
}

// The size of each segment's table after a segmented launch, written to mapped host memory (the scheduler
// reads it once the launch's event has fired).
__global__ void
k_gather_sizes(const seg_desc* segs, int32_t nseg, unsigned long long* out)
{
    for (int32_t s = static_cast<int32_t>(blockIdx.x * blockDim.x + threadIdx.x); s < nseg;
         s += static_cast<int32_t>(gridDim.x * blockDim.x))
    {
        out[s] = *reinterpret_cast<volatile unsigned long long*>(&segs[s].view.hdr->size);
    }
}

// Grow of a table without a host round trip: every element of src (its regular slots, then the two
// out-of-band slots of the tail group) is inserted into the empty, larger table dst by the bulk insert
// step, 32 consecutive slots of src per warp step.  src is read only; nothing else runs on either table
// meanwhile.
template <int KIND>
__global__ void __launch_bounds__(kThreads)
k_migrate(dview src, dview dst)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    constexpr int64_t sb = C::slot_bytes;
    const tile_lanes L;
    const int64_t regular = static_cast<int64_t>(src.num_groups) * C::slots_per_group;
    const int64_t n = regular + 2;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    step_counts c;
    for (int64_t base = warp * 32; base < n; base += nwarps * 32)
    {
        const int64_t i = base + L.lane;
        bool valid = false;
        K key = C::empty_key;
        V val{};
        if (i < regular)
        {
            key = __ldcs(reinterpret_cast<const K*>(src.slots + i * sb));
            valid = key < C::tomb_key; // neither never used nor erased
        }
        else if (i < n)
        {
            const int s = static_cast<int>(i - regular);
            valid = src.hdr->special_state[s] == 1u;
            key = s == 0 ? C::empty_key : C::tomb_key;
        }
        if constexpr (kind_traits<KIND>::is_map)
        {
            if (valid)
            {
                val = __ldcs(reinterpret_cast<const V*>(src.slots + i * sb + kind_traits<KIND>::val_offset));
            }
        }
        insert_kv_step<KIND>(dst, L, key, val, i, valid, nullptr, c);
    }
    unsigned long long v[2] = { c.done, c.refused };
    unsigned long long* const dst_counts[2] = { &dst.hdr->size, &dst.hdr->refused };
    block_add<2>(v, dst_counts);
}

sg_status
launch_migrate(int kind, const dview& src, const dview& dst, int grid_cap, cudaStream_t s)
{
    const int64_t slots = static_cast<int64_t>(src.num_groups) * (kGroupBytes / 4) + 2; // at most 32 per group
    const int64_t want = (slots + kThreads - 1) / kThreads;
    const int grid = static_cast<int>(want < grid_cap ? (want < 1 ? 1 : want) : grid_cap);
    switch (kind)
    {
        case 0:
            k_migrate<0><<<grid, kThreads, 0, s>>>(src, dst);
            break;
        case 1:
            k_migrate<1><<<grid, kThreads, 0, s>>>(src, dst);
            break;
        case 2:
            k_migrate<2><<<grid, kThreads, 0, s>>>(src, dst);
            break;
        case 3:
            k_migrate<3><<<grid, kThreads, 0, s>>>(src, dst);
            break;
        case 4:
            k_migrate<4><<<grid, kThreads, 0, s>>>(src, dst);
            break;
        case 5:
            k_migrate<5><<<grid, kThreads, 0, s>>>(src, dst);
            break;
        default:
            return SG_ERR_BAD_ARG;
    }
    SG_LAUNCH_CHECK();
    return SG_OK;
}

template <int KIND>
sg_status
launch_segments(int op, const seg_desc* segs, const int64_t* prefix, int32_t nseg, int64_t tiles, int grid_cap,
                cudaStream_t s)
{
    const int64_t want = (tiles * 32 / kSegTilesPerStep + kSegThreads - 1) / kSegThreads;
    const int grid = static_cast<int>(want < grid_cap ? (want < 1 ? 1 : want) : grid_cap);
    if (op == 0)
    {
        k_segments<KIND, 0><<<grid, kSegThreads, 0, s>>>(segs, prefix, nseg);
    }
    else if (op == 1)
    {
        k_segments<KIND, 1><<<grid, kSegThreads, 0, s>>>(segs, prefix, nseg);
    }
    else
    {
        k_segments<KIND, 2><<<grid, kSegThreads, 0, s>>>(segs, prefix, nseg);
    }
    SG_LAUNCH_CHECK();
    return SG_OK;
}

sg_status
launch_segments_kind(int kind, int op, const seg_desc* segs, const int64_t* prefix, int32_t nseg, int64_t tiles,
                     int grid_cap, cudaStream_t s)
{
    switch (kind)
    {
        case 0:
            return launch_segments<0>(op, segs, prefix, nseg, tiles, grid_cap, s);
        case 1:
            return launch_segments<1>(op, segs, prefix, nseg, tiles, grid_cap, s);
        case 2:
            return launch_segments<2>(op, segs, prefix, nseg, tiles, grid_cap, s);
        case 3:
            return launch_segments<3>(op, segs, prefix, nseg, tiles, grid_cap, s);
        case 4:
            return launch_segments<4>(op, segs, prefix, nseg, tiles, grid_cap, s);
        case 5:
            return launch_segments<5>(op, segs, prefix, nseg, tiles, grid_cap, s);
        default:
            return SG_ERR_BAD_ARG;
    }
}

} // namespace detail
} // namespace sg

using namespace sg::detail;

namespace
{

using clock_type = std::chrono::steady_clock;

constexpr int kSlotSegments = 4096; // segments one packed launch can carry
#ifndef SG_SERVER_POOL
#define SG_SERVER_POOL 1
#endif
// > 0: a budget / SG_SERVER_POOL_WARM_DIV block is mapped into the pool at creation (0: none).  Measured on the
// 1K-4M request stream (29 GB of tables at the end): a quarter of the 120 GB budget took the grows' table
// creation from 2.7-3.3 ms in all to 0.7 ms and the p99 from 470-522 us to 295 us; an eighth did not help
// (the tables outgrew it).
#ifndef SG_SERVER_POOL_WARM_DIV
#define SG_SERVER_POOL_WARM_DIV 4
#endif
// Request-size policy defaults (sg_server_set_policy): a table's run of same-operation requests with at
// least kDefaultDirectKeys keys runs as its own launches (cut into launches of at most kDefaultChunkKeys
// keys) on one of kDefaultDirectStreams low-priority streams, at most kDefaultMaxDirect such runs issued and
// not yet complete; smaller runs are packed into one segmented launch per operation on a high-priority
// stream.  Large runs of different tables on several streams overlap: one run of a table that fits in L2,
// or of a small request count, leaves most of the device idle (measured on the 1K-4M request stream:
// 1, 2 and 4 direct streams with 4-8 runs in flight gave 15.1, 12.7 and 11.0 ms with p99 434, 418 and
// 422 us).
constexpr int64_t kDefaultDirectKeys = int64_t{ 1 } << 16;
constexpr int64_t kDefaultChunkKeys = int64_t{ 1 } << 22;
constexpr int kDefaultMaxDirect = 8;
constexpr int kDefaultDirectStreams = 4;
constexpr int kMaxDirectLimit = 16;

struct request_rec
{
    sg_request r{};
    sg_status status = SG_OK;
    clock_type::time_point t_submit;
    clock_type::time_point t_done;
    bool done = false;
};

struct table_rec
{
    sg_unordered* h = nullptr;
    int64_t capacity = 0;
    int64_t max_size = 0;
    int64_t bytes = 0;
    int64_t size_bound = 0; // upper bound of size(): exact after a check, plus keys inserted since
    std::deque<int64_t> fifo;
    bool busy = false;
    bool grow_failed = false; // the last grow could not allocate: the waiting insert run is refused
    bool check_grow = false;  // a run completed: see whether the table should grow before its next inserts
};

// One segmented launch of small runs of one operation: its descriptors (device and pinned host), its
// completion event and what completes with it.
struct launch_slot
{
    seg_desc* d_segs = nullptr;
    int64_t* d_prefix = nullptr;
    seg_desc* h_segs = nullptr;
    int64_t* h_prefix = nullptr;
    unsigned long long* h_sizes = nullptr; // mapped: each segment's table size after an insert / erase launch
    unsigned long long* d_sizes = nullptr; // its device address
    cudaEvent_t done = nullptr;
    bool in_use = false;
    bool sizes = false; // h_sizes is filled by this launch
    std::vector<int64_t> tickets;
    std::vector<int32_t> tables;
    std::vector<int32_t> seg_tables; // table of each segment
};

// One table's run of large requests, launched chunk by chunk on one low-priority stream; or one table's
// grow (retire: the storage it replaced, released once the server is idle).
struct direct_unit
{
    cudaEvent_t done = nullptr;
    bool in_use = false;
    std::vector<int64_t> tickets;
    int32_t table = -1;
    sg_unordered* retire = nullptr;
    int64_t retire_bytes = 0;
    unsigned long long* h_size = nullptr; // pinned: the table's size after the run (insert / erase runs)
    bool size_valid = false;
    // a grow the grow thread has not launched yet (its event is not recorded): written by the grow thread,
    // read by the scheduler's event polling outside the lock
    std::atomic<bool> pending{ false };
};

// A grow handed to the grow thread: the new table's capacity and bytes, the storage it replaces.
struct grow_job
{
    int32_t table = -1;
    direct_unit* unit = nullptr;
    int64_t capacity = 0;
    int64_t max_size = 0;
    int64_t bytes = 0;
    sg_unordered* old = nullptr;
};

// What admit_insert_run decided for an insert run.
enum admit_result
{
    kAdmitRun,     // launch it
    kAdmitGrowing, // the table's grow was launched; the run waits for it
    kAdmitWait,    // no unit free for the grow; try again next round
    kAdmitRefused  // refused by the budget (its requests are complete)
};

} // namespace

struct sg_server
{
    int32_t kind = 0;
    int64_t budget = 0;
    int64_t used = 0;
    int grid_cap = 0;
    std::vector<cudaStream_t> hi_streams; // packed launches (greatest priority)
    std::vector<cudaStream_t> lo_streams; // large runs (least priority)
    unsigned long long* unit_sizes = nullptr; // pinned, one per direct unit
    cudaStream_t grow_stream = nullptr;   // grows (least priority)
    std::vector<std::pair<sg_unordered*, int64_t>> graveyard; // storage replaced by grows, and its bytes
    int next_hi = 0;
    int next_lo = 0;
    std::vector<launch_slot> slots;
    std::vector<direct_unit> units;
    int64_t direct_keys = kDefaultDirectKeys;
    int64_t chunk_keys = kDefaultChunkKeys;
    int max_direct = kDefaultMaxDirect;
    int direct_streams = kDefaultDirectStreams;
    bool grow_ahead_enabled = true;
    std::mutex m;
    std::condition_variable cv_work;
    std::condition_variable cv_done;
    std::unordered_map<int32_t, table_rec> tables;
    std::deque<request_rec> reqs; // index = ticket - ticket_base
    int64_t ticket_base = 0;
    std::vector<double> latencies_us;
    int64_t keys_done = 0;
    int64_t launches = 0;
    int64_t waves = 0;
    int64_t refused_budget = 0;
    int64_t rehashes = 0;
    double grow_host_us = 0.0;
    double max_grow_host_us = 0.0;
    clock_type::time_point t_first{}, t_last{};
    bool any_done = false;
    bool stop = false;
    bool stop_grows = false;
    bool paused = false;
    std::atomic<uint64_t> submissions{ 0 }; // bumped by every submit: wakes the scheduler's spin
    std::thread worker;
    std::thread grower; // creates and fills grown tables, so the scheduler keeps launching meanwhile
    std::deque<grow_job> grow_jobs;
    std::condition_variable cv_grow;
    int device = 0;
    // The tables' storage: a stream-ordered memory pool that keeps what it frees (release threshold
    // unlimited), so a grow after the first few takes its block from storage that earlier grows released
    // instead of mapping new memory.  Each allocation completes on its own idle stream before the table is
    // used elsewhere; a release follows a device synchronisation, as for every table.
    cudaMemPool_t pool = nullptr;
    cudaStream_t alloc_stream = nullptr;
    sg_allocator table_alloc{};
    double grow_thread_us = 0.0; // grow thread: time creating tables (allocation included)

    request_rec&
    rec(int64_t ticket)
    {
        return reqs[static_cast<size_t>(ticket - ticket_base)];
    }

    void run();
    void run_grows();
    void finish(const std::vector<int64_t>& tickets, clock_type::time_point now);
    bool complete_finished();
    bool any_in_flight() const;
    bool any_event_done();
    bool dispatch();
    admit_result admit_insert_run(int32_t table, table_rec& t, size_t take, int64_t run_keys);
    bool launch_direct(int32_t table, const std::vector<int64_t>& tickets);
    bool launch_packed(launch_slot& sl, int op, const std::vector<std::pair<int32_t, int64_t>>& run);
    direct_unit* free_unit();
    sg_status grow(int32_t table, table_rec& t, int64_t need, direct_unit& u, bool ahead = false);
    bool grow_ahead();
    void grow_done(const grow_job& job, sg_unordered* nh);
    void refuse_run(table_rec& t, size_t take);
    void release_graveyard();
};

namespace
{

void*
pool_alloc(size_t bytes, void* ctx)
{
    auto* srv = static_cast<sg_server*>(ctx);
    void* p = nullptr;
    if (cudaMallocFromPoolAsync(&p, bytes, srv->pool, srv->alloc_stream) != cudaSuccess ||
        cudaStreamSynchronize(srv->alloc_stream) != cudaSuccess)
    {
        cudaGetLastError();
        return nullptr;
    }
    return p;
}

void
pool_release(void* p, void* ctx)
{
    auto* srv = static_cast<sg_server*>(ctx);
    cudaFreeAsync(p, srv->alloc_stream); // the caller synchronised the device first
}

// A table of the server's kind and the given capacity, its storage from the server's pool (or the library's
// allocator when the pool could not be made).
sg_status
create_server_table(sg_server* srv, int64_t capacity, void* stream, sg_unordered** out)
{
    const sg_status st = srv->pool == nullptr
                                 ? sg_unordered_create(srv->kind, capacity, stream, out)
                                 : sg_unordered_create_with_allocator(srv->kind, capacity, 0, &srv->table_alloc, stream, out);
    if (st == SG_OK)
    {
        // the server's launches take keys until no slot is free
        sg::detail::unordered_accounting_off(*out);
    }
    return st;
}

int64_t
table_bytes(int32_t kind, int64_t capacity, int64_t* max_size)
{
    sg_geometry g{};
    if (sg_unordered_geometry_for(kind, capacity, &g) != SG_OK)
    {
        return -1;
    }
    *max_size = g.max_size;
    return g.storage_bytes;
}

dview
kernel_view(sg_unordered* h)
{
    sg_unordered_view v{};
    sg_unordered_view_of(h, &v);
    return dview{ static_cast<char*>(v.slots), static_cast<table_header*>(v.header),
                  static_cast<uint32_t>(v.num_groups), static_cast<uint32_t>(v.total_count), v.bucket_bits };
}

int
key_bytes_of_kind(int32_t kind)
{
    return (kind == SG_SET_U32 || kind == SG_MAP_U32_U32 || kind == SG_MAP_U32_U64) ? 4 : 8;
}

int
mapped_bytes_of_kind(int32_t kind)
{
    return kind == SG_MAP_U64_U32 || kind == SG_MAP_U32_U32 ? 4 : (kind == SG_MAP_U64_U64 || kind == SG_MAP_U32_U64 ? 8 : 0);
}

template <typename T>
T*
advance(T* p, int64_t bytes)
{
    return p == nullptr ? nullptr
                        : reinterpret_cast<T*>(reinterpret_cast<typename std::conditional<std::is_const<T>::value,
                                                                                          const char, char>::type*>(p) +
                                               bytes);
}

} // namespace

// Marks the requests done at `now`.  Caller holds the lock.
void
sg_server::finish(const std::vector<int64_t>& tickets, clock_type::time_point now)
{
    for (int64_t tk : tickets)
    {
        request_rec& r = rec(tk);
        r.done = true;
        r.t_done = now;
        latencies_us.push_back(std::chrono::duration<double, std::micro>(now - r.t_submit).count());
        keys_done += r.r.n;
    }
    t_last = now;
}

// Completes every launch whose event has fired: its requests are done and its tables free again.  Caller
// holds the lock.
bool
sg_server::complete_finished()
{
    bool any = false;
    for (auto& sl : slots)
    {
        if (!sl.in_use || cudaEventQuery(sl.done) != cudaSuccess)
        {
            continue;
        }
        finish(sl.tickets, clock_type::now());
        for (int32_t t : sl.tables)
        {
            auto it = tables.find(t);
            if (it != tables.end())
            {
                it->second.busy = false;
                it->second.check_grow = sl.sizes;
            }
        }
        if (sl.sizes)
        {
            // exact sizes: later segments of a table read the same final value
            for (size_t k = 0; k < sl.seg_tables.size(); ++k)
            {
                auto it = tables.find(sl.seg_tables[k]);
                if (it != tables.end())
                {
                    it->second.size_bound = static_cast<int64_t>(sl.h_sizes[k]);
                }
            }
        }
        sl.tickets.clear();
        sl.tables.clear();
        sl.seg_tables.clear();
        sl.sizes = false;
        sl.in_use = false;
        any = true;
    }
    for (auto& u : units)
    {
        if (!u.in_use || u.pending || cudaEventQuery(u.done) != cudaSuccess)
        {
            continue;
        }
        finish(u.tickets, clock_type::now());
        auto it = tables.find(u.table);
        if (it != tables.end())
        {
            it->second.busy = false;
            if (u.size_valid)
            {
                it->second.size_bound = static_cast<int64_t>(*u.h_size);
                it->second.check_grow = true;
            }
        }
        u.size_valid = false;
        if (u.retire != nullptr)
        {
            graveyard.push_back({ u.retire, u.retire_bytes });
            u.retire = nullptr;
            u.retire_bytes = 0;
        }
        u.tickets.clear();
        u.in_use = false;
        any = true;
    }
    return any;
}

bool
sg_server::any_in_flight() const
{
    for (const auto& sl : slots)
    {
        if (sl.in_use)
        {
            return true;
        }
    }
    for (const auto& u : units)
    {
        if (u.in_use)
        {
            return true;
        }
    }
    return false;
}

// Only the scheduler thread touches the events; safe without the lock.
bool
sg_server::any_event_done()
{
    for (auto& sl : slots)
    {
        if (sl.in_use && cudaEventQuery(sl.done) == cudaSuccess)
        {
            return true;
        }
    }
    for (auto& u : units)
    {
        if (u.in_use && !u.pending && cudaEventQuery(u.done) == cudaSuccess)
        {
            return true;
        }
    }
    return false;
}

// A direct unit not in use, or nullptr.
direct_unit*
sg_server::free_unit()
{
    for (auto& x : units)
    {
        if (!x.in_use)
        {
            return &x;
        }
    }
    return nullptr;
}

// Releases the storage that grows replaced.  cudaFree waits for the whole device, so this runs only when
// nothing of the server is in flight, or when the budget needs the bytes back.  Caller holds the lock.
void
sg_server::release_graveyard()
{
    for (auto& g : graveyard)
    {
        sg_unordered_destroy(g.first);
        used -= g.second;
    }
    graveyard.clear();
}

// Grows table t to the first doubling of its capacity under which `need` elements stay below 85 % of
// max_size(), when the budget allows.  Asynchronous: the grow thread creates the new table and fills it
// from the old one by k_migrate on the grow stream, the unit's event completes the grow, and until then
// the table is busy, so its requests keep their order; the scheduler goes on with other tables while the
// new storage is allocated.  The new bytes are counted at once, the old ones until the old storage is
// released.  Caller holds the lock; the table has nothing in flight.
sg_status
sg_server::grow(int32_t table, table_rec& t, int64_t need, direct_unit& u, bool ahead)
{
    const auto t0 = clock_type::now();
    int64_t cap = t.capacity;
    int64_t ms = 0;
    int64_t bytes = 0;
    do
    {
        cap *= 2;
        bytes = table_bytes(kind, cap, &ms);
        if (bytes < 0)
        {
            return SG_ERR_BUDGET;
        }
    } while (need > ms * 85 / 100);
    if (ahead && used + bytes > budget)
    {
        return SG_ERR_BUDGET; // growing ahead never waits for replaced storage to be released
    }
    if (used + bytes > budget && !graveyard.empty())
    {
        release_graveyard();
    }
    if (used + bytes > budget)
    {
        return SG_ERR_BUDGET;
    }
    grow_jobs.push_back(grow_job{ table, &u, cap, ms, bytes, t.h });
    u.tickets.clear();
    u.table = table;
    u.in_use = true;
    u.pending = true;
    used += bytes;
    t.busy = true;
    ++rehashes;
    cv_grow.notify_one();
    const double us = std::chrono::duration<double, std::micro>(clock_type::now() - t0).count();
    grow_host_us += us;
    max_grow_host_us = us > max_grow_host_us ? us : max_grow_host_us;
    return SG_OK;
}

// The grow thread: for each job, the new table and the migrate launch on the grow stream, then the unit's
// event; the job's table is busy meanwhile, so nothing else touches its storage.
void
sg_server::run_grows()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lock(m);
    while (true)
    {
        cv_grow.wait(lock, [&] { return stop_grows || !grow_jobs.empty(); });
        if (grow_jobs.empty())
        {
            return;
        }
        const grow_job job = grow_jobs.front();
        grow_jobs.pop_front();
        lock.unlock();
        sg_unordered* nh = nullptr;
        const auto c0 = clock_type::now();
        sg_status st = create_server_table(this, job.capacity, grow_stream, &nh);
        const double create_us = std::chrono::duration<double, std::micro>(clock_type::now() - c0).count();
        if (st == SG_OK)
        {
            st = launch_migrate(kind, kernel_view(job.old), kernel_view(nh), grid_cap, grow_stream);
            if (st == SG_OK && cudaEventRecord(job.unit->done, grow_stream) != cudaSuccess)
            {
                st = SG_ERR_CUDA;
            }
            if (st != SG_OK)
            {
                cudaStreamSynchronize(grow_stream);
                sg_unordered_destroy(nh);
                nh = nullptr;
            }
        }
        cudaGetLastError();
        lock.lock();
        grow_thread_us += create_us;
        grow_done(job, nh);
        lock.unlock();
        submissions.fetch_add(1, std::memory_order_release); // wakes the scheduler's spin
        cv_work.notify_one();
        lock.lock();
    }
}

// A grow job's outcome.  Launched: the table takes the new storage and the unit completes with its event,
// the old storage then retiring.  Failed: the bytes go back, the table is free again and its waiting insert
// run is refused.  Caller holds the lock.
void
sg_server::grow_done(const grow_job& job, sg_unordered* nh)
{
    direct_unit& u = *job.unit;
    table_rec& t = tables[job.table];
    if (nh != nullptr)
    {
        u.retire = job.old;
        u.retire_bytes = t.bytes;
        u.pending = false;
        t.h = nh;
        t.capacity = job.capacity;
        t.max_size = job.max_size;
        t.bytes = job.bytes;
    }
    else
    {
        used -= job.bytes;
        --rehashes;
        u.pending = false;
        u.in_use = false;
        t.busy = false;
        t.grow_failed = true;
    }
}

// Growing ahead: a table whose last insert / erase run left it more than half full (its exact size, read
// back with the run) and that has no request waiting grows to the next doubling now, while it is idle, so an
// insert that arrives later does not wait for the rehash.  Only within the budget as it stands.  Caller holds
// the lock.  Returns true when a grow was launched.
bool
sg_server::grow_ahead()
{
    bool any = false;
    for (auto& kv : tables)
    {
        table_rec& t = kv.second;
        if (!t.check_grow || t.busy || !t.fifo.empty())
        {
            continue;
        }
        t.check_grow = false;
        if (t.size_bound * 2 <= t.max_size)
        {
            continue;
        }
        direct_unit* u = free_unit();
        if (u == nullptr)
        {
            t.check_grow = true;
            break;
        }
        any = grow(kv.first, t, t.size_bound * 17 / 10, *u, true) == SG_OK || any;
    }
    return any;
}

// Completes the first `take` requests of table t with SG_ERR_BUDGET (refused; nothing spills).  Caller holds
// the lock.
void
sg_server::refuse_run(table_rec& t, size_t take)
{
    const auto now = clock_type::now();
    for (size_t k = 0; k < take; ++k)
    {
        request_rec& r = rec(t.fifo.front());
        r.status = SG_ERR_BUDGET;
        r.done = true;
        r.t_done = now;
        ++refused_budget;
        t.fifo.pop_front();
    }
    cv_done.notify_all();
}

// Before an insert run of `take` requests and run_keys keys: if the run could pass 85 % of max_size(), the
// table's exact size is read and, if that does not rule it out, the table grows first (the run waits for
// the grow).  When the budget does not allow the grow, the run's requests complete with SG_ERR_BUDGET
// (nothing spills).  Caller holds the lock.
admit_result
sg_server::admit_insert_run(int32_t table, table_rec& t, size_t take, int64_t run_keys)
{
    if (t.grow_failed)
    {
        // the grow this run waited for could not allocate its table
        t.grow_failed = false;
        refuse_run(t, take);
        return kAdmitRefused;
    }
    if (t.size_bound + run_keys > t.max_size * 85 / 100)
    {
        int64_t exact = 0;
        if (sg_unordered_size(t.h, nullptr, &exact) == SG_OK)
        {
            t.size_bound = exact;
        }
        if (t.size_bound + run_keys > t.max_size * 85 / 100)
        {
            direct_unit* u = free_unit();
            if (u == nullptr)
            {
                return kAdmitWait;
            }
            if (grow(table, t, t.size_bound + run_keys, *u) == SG_OK)
            {
                return kAdmitGrowing;
            }
            refuse_run(t, take);
            return kAdmitRefused;
        }
    }
    t.size_bound += run_keys;
    return kAdmitRun;
}

// A table's run of large requests: each request is cut into launches of at most chunk_keys keys on one
// low-priority stream (in request order, so the table sees them in submission order); the unit's event
// completes the run.  Caller holds the lock and has checked that a unit is free.
bool
sg_server::launch_direct(int32_t table, const std::vector<int64_t>& tickets)
{
    direct_unit* u = free_unit();
    if (u == nullptr)
    {
        return false;
    }
    sg_unordered* h = tables[table].h;
    const int nlo = direct_streams < static_cast<int>(lo_streams.size()) ? direct_streams
                                                                        : static_cast<int>(lo_streams.size());
    next_lo = (next_lo + 1) % nlo;
    cudaStream_t s = lo_streams[next_lo];
    const int kb = key_bytes_of_kind(kind);
    const int mb = mapped_bytes_of_kind(kind);
    bool ok = true;
    for (int64_t tk : tickets)
    {
        const sg_request& r = rec(tk).r;
        for (int64_t off = 0; off < r.n && ok; off += chunk_keys)
        {
            const int64_t len = r.n - off < chunk_keys ? r.n - off : chunk_keys;
            sg_status st = SG_OK;
            if (r.op == SG_SERVER_INSERT)
            {
                st = sg_unordered_insert_kv(h, advance(r.keys, off * kb), advance(r.mapped, off * mb), len,
                                            advance(r.out_flags, off), s);
            }
            else if (r.op == SG_SERVER_FIND)
            {
                st = sg_unordered_find(h, advance(r.keys, off * kb), len, advance(r.out_mapped, off * mb),
                                       advance(r.out_flags, off), s);
            }
            else
            {
                st = sg_unordered_erase(h, advance(r.keys, off * kb), len, advance(r.out_flags, off), s);
            }
            ok = st == SG_OK;
            ++launches;
        }
        if (!ok)
        {
            rec(tk).status = SG_ERR_CUDA;
        }
    }
    const int run_op = tickets.empty() ? SG_SERVER_FIND : rec(tickets.front()).r.op;
    u->size_valid = false;
    if (ok && run_op != SG_SERVER_FIND)
    {
        u->size_valid = cudaMemcpyAsync(u->h_size, &kernel_view(h).hdr->size, sizeof(unsigned long long),
                                        cudaMemcpyDeviceToHost, s) == cudaSuccess;
    }
    cudaEventRecord(u->done, s);
    u->tickets = tickets;
    u->table = table;
    u->in_use = true;
    return true;
}

// One segmented launch of small runs of operation `op` on a high-priority stream.  Caller holds the lock.
bool
sg_server::launch_packed(launch_slot& sl, int op, const std::vector<std::pair<int32_t, int64_t>>& run)
{
    int64_t tiles = 0;
    int nseg = 0;
    for (const auto& tr : run)
    {
        const request_rec& r = rec(tr.second);
        seg_desc& d = sl.h_segs[nseg];
        d.view = kernel_view(tables[tr.first].h);
        d.in0 = r.r.keys;
        d.in1 = r.r.mapped;
        d.out_vals = r.r.out_mapped;
        d.out_flags = r.r.out_flags;
        d.n = r.r.n;
        sl.h_prefix[nseg] = tiles;
        tiles += (r.r.n + 31) / 32;
        sl.tickets.push_back(tr.second);
        sl.seg_tables.push_back(tr.first);
        if (sl.tables.empty() || sl.tables.back() != tr.first)
        {
            sl.tables.push_back(tr.first);
        }
        ++nseg;
    }
    sl.h_prefix[nseg] = tiles;
    cudaStream_t s = hi_streams[next_hi];
    next_hi = (next_hi + 1) % static_cast<int>(hi_streams.size());
    bool ok = cudaMemcpyAsync(sl.d_segs, sl.h_segs, sizeof(seg_desc) * nseg, cudaMemcpyHostToDevice, s) ==
                      cudaSuccess &&
              cudaMemcpyAsync(sl.d_prefix, sl.h_prefix, sizeof(int64_t) * (nseg + 1), cudaMemcpyHostToDevice, s) ==
                      cudaSuccess;
    ok = ok && launch_segments_kind(kind, op, sl.d_segs, sl.d_prefix, nseg, tiles, grid_cap, s) == SG_OK;
    ++launches;
    if (ok && op != SG_SERVER_FIND)
    {
        k_gather_sizes<<<(nseg + 255) / 256, 256, 0, s>>>(sl.d_segs, nseg, sl.d_sizes);
        sl.sizes = cudaGetLastError() == cudaSuccess;
    }
    cudaEventRecord(sl.done, s);
    sl.in_use = true;
    if (!ok)
    {
        for (int64_t tk : sl.tickets)
        {
            rec(tk).status = SG_ERR_CUDA;
        }
    }
    return true;
}

// One scheduling round.  Tables with pending requests and nothing in flight are taken oldest request
// first; each contributes its run of consecutive same-operation requests.  A run of at least direct_keys
// keys becomes a direct unit while fewer than max_direct are in flight (else the table waits); smaller
// runs join the round's packed launch of their operation, when a launch slot is free for it.  Caller
// holds the lock.  Returns true when something was launched.
bool
sg_server::dispatch()
{
    std::vector<std::pair<int64_t, int32_t>> cand;
    for (auto& kv : tables)
    {
        if (!kv.second.busy && !kv.second.fifo.empty())
        {
            cand.push_back({ kv.second.fifo.front(), kv.first });
        }
    }
    if (cand.empty())
    {
        return grow_ahead_enabled && grow_ahead();
    }
    std::sort(cand.begin(), cand.end());
    int direct_busy = 0;
    for (const auto& u : units)
    {
        direct_busy += u.in_use && u.retire == nullptr ? 1 : 0; // grows do not count
    }
    launch_slot* op_slot[3] = { nullptr, nullptr, nullptr };
    std::vector<std::pair<int32_t, int64_t>> packed[3];
    int packed_segs[3] = { 0, 0, 0 };
    bool launched = false;
    for (const auto& c : cand)
    {
        table_rec& t = tables[c.second];
        const int op = rec(t.fifo.front()).r.op;
        size_t take = 0;
        int64_t run_keys = 0;
        while (take < t.fifo.size() && rec(t.fifo[take]).r.op == op && take < static_cast<size_t>(kSlotSegments))
        {
            run_keys += rec(t.fifo[take]).r.n;
            ++take;
        }
        const bool big = run_keys >= direct_keys;
        if (big && direct_busy >= max_direct)
        {
            continue;
        }
        if (!big)
        {
            if (packed_segs[op] + static_cast<int>(take) > kSlotSegments)
            {
                continue;
            }
            if (op_slot[op] == nullptr)
            {
                for (auto& sl : slots)
                {
                    if (!sl.in_use && &sl != op_slot[0] && &sl != op_slot[1] && &sl != op_slot[2])
                    {
                        op_slot[op] = &sl;
                        break;
                    }
                }
                if (op_slot[op] == nullptr)
                {
                    continue;
                }
            }
        }
        if (op == SG_SERVER_INSERT)
        {
            const admit_result a = admit_insert_run(c.second, t, take, run_keys);
            if (a == kAdmitGrowing)
            {
                launched = true;
            }
            if (a != kAdmitRun)
            {
                continue;
            }
        }
        std::vector<int64_t> tk;
        tk.reserve(take);
        for (size_t k = 0; k < take; ++k)
        {
            tk.push_back(t.fifo.front());
            t.fifo.pop_front();
        }
        t.busy = true;
        if (big)
        {
            launch_direct(c.second, tk);
            ++direct_busy;
            launched = true;
        }
        else
        {
            for (int64_t x : tk)
            {
                packed[op].push_back({ c.second, x });
            }
            packed_segs[op] += static_cast<int>(take);
        }
    }
    for (int op = 0; op < 3; ++op)
    {
        if (!packed[op].empty())
        {
            launch_packed(*op_slot[op], op, packed[op]);
            launched = true;
        }
    }
    if (launched)
    {
        ++waves;
    }
    if (grow_ahead_enabled && grow_ahead())
    {
        launched = true;
    }
    return launched;
}

void
sg_server::run()
{
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lock(m);
    while (true)
    {
        if (complete_finished())
        {
            cv_done.notify_all();
        }
        const bool launched = !paused && dispatch();
        const bool in_flight = any_in_flight();
        if (!in_flight && !graveyard.empty())
        {
            release_graveyard();
        }
        if (stop && !in_flight)
        {
            break;
        }
        if (in_flight)
        {
            // Spin outside the lock until a launch completes or a request arrives; only this thread
            // touches the events.  After ~200 us of spinning, yield the core between polls.
            const uint64_t seen = submissions.load(std::memory_order_acquire);
            lock.unlock();
            const auto t0 = clock_type::now();
            while (!any_event_done() && submissions.load(std::memory_order_acquire) == seen)
            {
                if (clock_type::now() - t0 > std::chrono::microseconds(200))
                {
                    std::this_thread::yield();
                }
            }
            lock.lock();
        }
        else if (!launched)
        {
            cv_work.wait_for(lock, std::chrono::milliseconds(5));
        }
    }
    cv_done.notify_all();
}

extern "C" {

sg_status
sg_server_create(int32_t kind, int64_t hbm_budget_bytes, int32_t n_streams, int32_t n_slots, sg_server** out)
{
    if (out == nullptr || kind < SG_SET_U32 || kind > SG_MAP_U32_U64 || hbm_budget_bytes <= 0 || n_streams < 1 ||
        n_streams > 64 || n_slots < 1 || n_slots > 256)
    {
        return SG_ERR_BAD_ARG;
    }
    *out = nullptr;
    auto* srv = new (std::nothrow) sg_server{};
    if (srv == nullptr)
    {
        return SG_ERR_OOM;
    }
    srv->kind = kind;
    srv->budget = hbm_budget_bytes;
    cudaGetDevice(&srv->device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, srv->device);
    srv->grid_cap = sms * 8;
    int least = 0, greatest = 0;
    cudaDeviceGetStreamPriorityRange(&least, &greatest);
    srv->hi_streams.resize(n_streams);
    for (auto& s : srv->hi_streams)
    {
        cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, greatest);
    }
    srv->lo_streams.resize(n_streams);
    for (auto& s : srv->lo_streams)
    {
        cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, least);
    }
    cudaStreamCreateWithPriority(&srv->grow_stream, cudaStreamNonBlocking, least);
#if SG_SERVER_POOL
    {
        cudaMemPoolProps props{};
        props.allocType = cudaMemAllocationTypePinned;
        props.location.type = cudaMemLocationTypeDevice;
        props.location.id = srv->device;
        if (cudaMemPoolCreate(&srv->pool, &props) == cudaSuccess)
        {
            unsigned long long keep = ~0ull;
            cudaMemPoolSetAttribute(srv->pool, cudaMemPoolAttrReleaseThreshold, &keep);
            cudaStreamCreateWithFlags(&srv->alloc_stream, cudaStreamNonBlocking);
            srv->table_alloc = sg_allocator{ &pool_alloc, &pool_release, srv, nullptr };
#if SG_SERVER_POOL_WARM_DIV > 0
            // map part of the budget into the pool up front, so the first grows do not map memory
            void* warm = nullptr;
            if (cudaMallocFromPoolAsync(&warm, static_cast<size_t>(hbm_budget_bytes / SG_SERVER_POOL_WARM_DIV), srv->pool,
                                        srv->alloc_stream) == cudaSuccess)
            {
                cudaFreeAsync(warm, srv->alloc_stream);
            }
            cudaStreamSynchronize(srv->alloc_stream);
            cudaGetLastError();
#endif
        }
        else
        {
            srv->pool = nullptr;
            cudaGetLastError();
        }
    }
#endif
    srv->units = std::vector<direct_unit>(kMaxDirectLimit);
    if (cudaMallocHost(&srv->unit_sizes, sizeof(unsigned long long) * kMaxDirectLimit) != cudaSuccess)
    {
        cudaGetLastError();
        sg_server_destroy(srv);
        return SG_ERR_OOM;
    }
    for (int k = 0; k < kMaxDirectLimit; ++k)
    {
        srv->units[k].h_size = srv->unit_sizes + k;
    }
    for (auto& u : srv->units)
    {
        if (cudaEventCreateWithFlags(&u.done, cudaEventDisableTiming) != cudaSuccess)
        {
            cudaGetLastError();
            sg_server_destroy(srv);
            return SG_ERR_OOM;
        }
    }
    srv->slots.resize(n_slots);
    for (auto& sl : srv->slots)
    {
        if (sg::detail::dev_malloc(&sl.d_segs, sizeof(seg_desc) * kSlotSegments) != cudaSuccess ||
            sg::detail::dev_malloc(&sl.d_prefix, sizeof(int64_t) * (kSlotSegments + 1)) != cudaSuccess ||
            cudaMallocHost(&sl.h_segs, sizeof(seg_desc) * kSlotSegments) != cudaSuccess ||
            cudaMallocHost(&sl.h_prefix, sizeof(int64_t) * (kSlotSegments + 1)) != cudaSuccess ||
            cudaHostAlloc(&sl.h_sizes, sizeof(unsigned long long) * kSlotSegments, cudaHostAllocMapped) != cudaSuccess ||
            cudaHostGetDevicePointer(reinterpret_cast<void**>(&sl.d_sizes), sl.h_sizes, 0) != cudaSuccess ||
            cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming) != cudaSuccess)
        {
            cudaGetLastError();
            sg_server_destroy(srv);
            return SG_ERR_OOM;
        }
    }
    srv->grower = std::thread([srv] { srv->run_grows(); });
    srv->worker = std::thread([srv] { srv->run(); });
    *out = srv;
    return SG_OK;
}

sg_status
sg_server_destroy(sg_server* srv)
{
    if (srv == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    {
        std::lock_guard<std::mutex> lock(srv->m);
        srv->stop = true;
    }
    srv->cv_work.notify_all();
    if (srv->worker.joinable())
    {
        srv->worker.join(); // returns once nothing is in flight, pending grows included
    }
    {
        std::lock_guard<std::mutex> lock(srv->m);
        srv->stop_grows = true;
    }
    srv->cv_grow.notify_all();
    if (srv->grower.joinable())
    {
        srv->grower.join();
    }
    cudaDeviceSynchronize();
    srv->release_graveyard();
    for (auto& kv : srv->tables)
    {
        sg_unordered_destroy(kv.second.h);
    }
    srv->tables.clear();
    if (srv->alloc_stream != nullptr)
    {
        cudaStreamSynchronize(srv->alloc_stream);
        cudaStreamDestroy(srv->alloc_stream);
    }
    if (srv->pool != nullptr)
    {
        cudaMemPoolDestroy(srv->pool);
    }
    for (auto& sl : srv->slots)
    {
        sg::detail::dev_free(sl.d_segs);
        sg::detail::dev_free(sl.d_prefix);
        if (sl.h_segs != nullptr)
        {
            cudaFreeHost(sl.h_segs);
        }
        if (sl.h_prefix != nullptr)
        {
            cudaFreeHost(sl.h_prefix);
        }
        if (sl.h_sizes != nullptr)
        {
            cudaFreeHost(sl.h_sizes);
        }
        if (sl.done != nullptr)
        {
            cudaEventDestroy(sl.done);
        }
    }
    for (auto& u : srv->units)
    {
        if (u.done != nullptr)
        {
            cudaEventDestroy(u.done);
        }
    }
    if (srv->grow_stream != nullptr)
    {
        cudaStreamDestroy(srv->grow_stream);
    }
    if (srv->unit_sizes != nullptr)
    {
        cudaFreeHost(srv->unit_sizes);
    }
    for (auto* v : { &srv->hi_streams, &srv->lo_streams })
    {
        for (auto& s : *v)
        {
            if (s != nullptr)
            {
                cudaStreamDestroy(s);
            }
        }
    }
    delete srv;
    return SG_OK;
}

sg_status
sg_server_set_policy(sg_server* srv, int64_t direct_keys, int64_t chunk_keys, int32_t max_direct,
                     int32_t direct_streams)
{
    if (srv == nullptr || direct_keys < 1 || chunk_keys < 1 || max_direct < 1 || max_direct > kMaxDirectLimit ||
        direct_streams < 1 || direct_streams > static_cast<int32_t>(srv->lo_streams.size()))
    {
        return SG_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lock(srv->m);
    srv->direct_keys = direct_keys;
    srv->chunk_keys = chunk_keys;
    srv->max_direct = max_direct;
    srv->direct_streams = direct_streams;
    return SG_OK;
}

sg_status
sg_server_set_grow_ahead(sg_server* srv, int32_t enabled)
{
    if (srv == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lock(srv->m);
    srv->grow_ahead_enabled = enabled != 0;
    return SG_OK;
}

sg_status
sg_server_admit_table(sg_server* srv, int32_t table, int64_t capacity)
{
    if (srv == nullptr || table < 0 || capacity <= 0)
    {
        return SG_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lock(srv->m);
    if (srv->tables.count(table) != 0)
    {
        return SG_ERR_BAD_ARG;
    }
    int64_t ms = 0;
    const int64_t bytes = table_bytes(srv->kind, capacity, &ms);
    if (bytes < 0)
    {
        return SG_ERR_BAD_ARG;
    }
    if (srv->used + bytes > srv->budget)
    {
        return SG_ERR_BUDGET;
    }
    table_rec t;
    const sg_status st = create_server_table(srv, capacity, nullptr, &t.h);
    if (st != SG_OK)
    {
        return st;
    }
    if (cudaDeviceSynchronize() != cudaSuccess)
    {
        sg_unordered_destroy(t.h);
        return SG_ERR_CUDA;
    }
    t.capacity = capacity;
    t.max_size = ms;
    t.bytes = bytes;
    srv->used += bytes;
    srv->tables.emplace(table, std::move(t));
    return SG_OK;
}

sg_status
sg_server_drop_table(sg_server* srv, int32_t table)
{
    if (srv == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    std::unique_lock<std::mutex> lock(srv->m);
    auto it = srv->tables.find(table);
    if (it == srv->tables.end())
    {
        return SG_ERR_BAD_ARG;
    }
    srv->cv_done.wait(lock, [&] { return !it->second.busy && it->second.fifo.empty(); });
    sg_unordered_destroy(it->second.h);
    srv->used -= it->second.bytes;
    srv->tables.erase(it);
    return SG_OK;
}

sg_status
sg_server_submit_many(sg_server* srv, const sg_request* reqs, int32_t n, int64_t* out_tickets)
{
    if (srv == nullptr || (n > 0 && (reqs == nullptr || out_tickets == nullptr)) || n < 0)
    {
        return SG_ERR_BAD_ARG;
    }
    for (int32_t k = 0; k < n; ++k)
    {
        const sg_request& r = reqs[k];
        if (r.n < 0 || (r.n > 0 && r.keys == nullptr) || r.op < SG_SERVER_INSERT || r.op > SG_SERVER_ERASE)
        {
            return SG_ERR_BAD_ARG;
        }
    }
    {
        std::lock_guard<std::mutex> lock(srv->m);
        if (srv->stop)
        {
            return SG_ERR_BAD_ARG;
        }
        for (int32_t k = 0; k < n; ++k)
        {
            if (srv->tables.find(reqs[k].table) == srv->tables.end())
            {
                return SG_ERR_BAD_ARG;
            }
        }
        const auto now = clock_type::now();
        for (int32_t k = 0; k < n; ++k)
        {
            const int64_t ticket = srv->ticket_base + static_cast<int64_t>(srv->reqs.size());
            request_rec r;
            r.r = reqs[k];
            r.t_submit = now;
            if (!srv->any_done)
            {
                srv->t_first = now;
                srv->any_done = true;
            }
            if (reqs[k].n == 0)
            {
                r.done = true;
                r.t_done = now;
                srv->reqs.push_back(r);
            }
            else
            {
                srv->reqs.push_back(r);
                srv->tables[reqs[k].table].fifo.push_back(ticket);
            }
            out_tickets[k] = ticket;
        }
    }
    srv->submissions.fetch_add(1, std::memory_order_release);
    srv->cv_work.notify_one();
    return SG_OK;
}

sg_status
sg_server_submit(sg_server* srv, const sg_request* req, int64_t* out_ticket)
{
    return sg_server_submit_many(srv, req, req != nullptr ? 1 : 0, out_ticket);
}

sg_status
sg_server_set_paused(sg_server* srv, int32_t paused)
{
    if (srv == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    {
        std::lock_guard<std::mutex> lock(srv->m);
        srv->paused = paused != 0;
    }
    srv->cv_work.notify_all();
    return SG_OK;
}

sg_status
sg_server_wait(sg_server* srv, int64_t ticket, int32_t timeout_ms, sg_status* out_request_status)
{
    if (srv == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    std::unique_lock<std::mutex> lock(srv->m);
    if (ticket < srv->ticket_base || ticket >= srv->ticket_base + static_cast<int64_t>(srv->reqs.size()))
    {
        return SG_ERR_BAD_ARG;
    }
    const bool ok = srv->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 3600000 : timeout_ms),
                                          [&] { return srv->rec(ticket).done; });
    if (!ok)
    {
        return SG_ERR_RETRY_EXHAUSTED;
    }
    if (out_request_status != nullptr)
    {
        *out_request_status = srv->rec(ticket).status;
    }
    return SG_OK;
}

sg_status
sg_server_drain(sg_server* srv, int32_t timeout_ms)
{
    if (srv == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    std::unique_lock<std::mutex> lock(srv->m);
    const bool ok = srv->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms < 0 ? 3600000 : timeout_ms), [&] {
        for (const auto& r : srv->reqs)
        {
            if (!r.done)
            {
                return false;
            }
        }
        return true;
    });
    return ok ? SG_OK : SG_ERR_RETRY_EXHAUSTED;
}

sg_status
sg_server_get_stats(sg_server* srv, sg_server_stats* out)
{
    if (srv == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lock(srv->m);
    std::vector<double> v = srv->latencies_us;
    std::sort(v.begin(), v.end());
    auto pct = [&](double p) {
        if (v.empty())
        {
            return 0.0;
        }
        size_t k = static_cast<size_t>(p * static_cast<double>(v.size() - 1) + 0.5);
        return v[std::min(k, v.size() - 1)];
    };
    out->requests_done = static_cast<int64_t>(v.size());
    out->keys_done = srv->keys_done;
    out->p50_us = pct(0.50);
    out->p99_us = pct(0.99);
    out->max_us = v.empty() ? 0.0 : v.back();
    const double span = srv->any_done ? std::chrono::duration<double>(srv->t_last - srv->t_first).count() : 0.0;
    out->keys_per_s = span > 0 ? static_cast<double>(srv->keys_done) / span : 0.0;
    out->launches = srv->launches;
    out->waves = srv->waves;
    out->refused_budget = srv->refused_budget;
    out->rehashes = srv->rehashes;
    out->hbm_used_bytes = srv->used;
    out->grow_host_us = srv->grow_host_us;
    out->max_grow_host_us = srv->max_grow_host_us;
    out->grow_create_us = srv->grow_thread_us;
    return SG_OK;
}

sg_status
sg_server_request_latency(sg_server* srv, int64_t ticket, double* out_us)
{
    if (srv == nullptr || out_us == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    std::lock_guard<std::mutex> lock(srv->m);
    if (ticket < srv->ticket_base || ticket >= srv->ticket_base + static_cast<int64_t>(srv->reqs.size()))
    {
        return SG_ERR_BAD_ARG;
    }
    const request_rec& r = srv->rec(ticket);
    if (!r.done)
    {
        return SG_ERR_RETRY_EXHAUSTED;
    }
    *out_us = std::chrono::duration<double, std::micro>(r.t_done - r.t_submit).count();
    return SG_OK;
}

sg_status
sg_server_table_view(sg_server* srv, int32_t table, sg_unordered_view* out)
{
    if (srv == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    std::unique_lock<std::mutex> lock(srv->m);
    auto it = srv->tables.find(table);
    if (it == srv->tables.end())
    {
        return SG_ERR_BAD_ARG;
    }
    // a grow in flight replaces the storage: the view is taken once the table has settled
    srv->cv_done.wait(lock, [&] { return !it->second.busy && it->second.fifo.empty(); });
    return sg_unordered_view_of(it->second.h, out);
}

sg_status
sg_server_table_size(sg_server* srv, int32_t table, int64_t* out_size)
{
    if (srv == nullptr || out_size == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    std::unique_lock<std::mutex> lock(srv->m);
    auto it = srv->tables.find(table);
    if (it == srv->tables.end())
    {
        return SG_ERR_BAD_ARG;
    }
    srv->cv_done.wait(lock, [&] { return !it->second.busy && it->second.fifo.empty(); });
    return sg_unordered_size(it->second.h, nullptr, out_size);
}

} // extern "C"

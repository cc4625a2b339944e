// unordered_set / unordered_map for GB300 (sm_103a): bulk kernels and the C ABI.
//
// Replaces the reference's table core (src/stdgpu/impl/unordered_base.cuh,
// src/stdgpu/impl/unordered_base_detail.cuh): a bucket array plus a linked
// excess list guarded by per-slot spin locks becomes open addressing over
// 128-byte probe groups (layout in include/stdgpu_gb300/detail/layout.cuh).
//
// Bulk kernels are tile-cooperative: 4 lanes own one key and read its
// 128-byte probe group as one request (one 32-byte sector per lane, 256-bit
// loads through L2); a warp holds 32 keys and each tile issues the home-group
// loads of its 4 keys before resolving them.  Slots are claimed lock-free with
// one compare-and-swap on the key word; counters are reduced per block and
// added once per block.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <new>
#include <type_traits>
#include <vector>

#include "sg_internal.cuh"
#include "stdgpu_gb300.h"
#include "stdgpu_gb300/detail/layout.cuh"
#include "stdgpu_gb300/device.cuh"
#include "bulk_stage.cuh"
#include "table_core.cuh"

namespace sg
{
namespace detail
{

std::atomic<long long> g_launches{ 0 };

SG_D bool
bit_set(const uint32_t* words, int64_t i)
{
    return (__ldcg(words + (i >> 5)) >> (i & 31)) & 1u;
}

// ---------------------------------------------------------------- kernels

// Fills every slot with the never-used marker and the slots at or above total_count with the erased
// marker; resets the header.  clear(): unordered_base_detail.cuh:1220-1252 (one launch instead of four).
template <int KIND>
__global__ void __launch_bounds__(kThreads)
k_init(dview t)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    constexpr int G = C::slots_per_group;
    const int64_t lanes_total = (t.num_groups + 1) * (kGroupBytes / 16); // 16-byte units, tail group included
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    uint4* base = reinterpret_cast<uint4*>(t.slots);
    for (int64_t u = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; u < lanes_total; u += stride)
    {
        const int64_t first = u * C::slots_per_lane;
        if (first + C::slots_per_lane <= t.total || first >= t.num_groups * G)
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
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        t.hdr->size = 0;
        t.hdr->refused = 0;
        t.hdr->tombstones = 0;
        t.hdr->excess_used = 0;
        t.hdr->special_state[0] = 0;
        t.hdr->special_state[1] = 0;
        t.hdr->error = 0;
        t.hdr->count = 0;
    }
}

// Bulk insert: src/stdgpu/impl/unordered_base_detail.cuh:996-1017 (insert_value :470-495).
template <int KIND, bool AOS>
__global__ void __launch_bounds__(kThreads, SG_BULK_MIN_BLOCKS)
k_insert(dview t, const void* in0, const void* in1, int64_t n, uint8_t* out_flags, const uint64_t* hashes,
         const unsigned int* gate)
{
    // a gated launch (the fallback of a partitioned insert) runs only when its gate word is set
    if (gate != nullptr && *gate == 0u)
    {
        return;
    }
    const tile_lanes L;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    step_counts c;
    for (int64_t base = warp * 32; base < n; base += nwarps * 32)
    {
        const int64_t i = base + L.lane;
        insert_step<KIND, AOS>(t, L, in0, in1, i, i < n, out_flags, c, hashes);
    }
    if (c.retry != 0)
    {
        atomicOr(&t.hdr->error, kErrRetry);
    }
    // size += inserted; refused += refused; tombstones -= reused
    unsigned long long v[3] = { c.done, c.refused, 0ull - c.reused };
    unsigned long long* const dst[3] = { &t.hdr->size, &t.hdr->refused, &t.hdr->tombstones };
    block_add<3>(v, dst);
}

// ---------------------------------------------------------------- partitioned bulk insert
// When a bulk insert brings many keys per probe group of a table far larger than L2, the keys are first
// split into P partitions by home-group range (the top bits of the reference bucket) and written as
// value_type elements into a scratch array, partition after partition; k_insert then walks that array
// in order, so the warps in flight work inside one or two partitions' groups (tens of MB) at a time and
// each group line is read from DRAM about once instead of once per key.  Element order inside a
// partition is arbitrary, as is the order among duplicates of one key in a single bulk insert.

constexpr int kPartMax = 256;
#ifndef SG_PART_PER
#define SG_PART_PER 4
#endif
constexpr int kPartPer = SG_PART_PER; // elements per thread per scatter round
// the same for elements of at most 8 bytes (bare keys of an erase, set keys): a tile of more elements gives
// each partition's run more bytes per tile and spreads the tile's fixed steps over more elements
#ifndef SG_PART_PER_NARROW
#define SG_PART_PER_NARROW 4
#endif
template <int KIND>
constexpr int part_per = kind_consts<KIND>::slot_bytes <= 8 ? SG_PART_PER_NARROW : kPartPer;

template <int KIND, bool AOS>
SG_D typename kind_consts<KIND>::K
load_key(const void* in0, int64_t i)
{
    using K = typename kind_consts<KIND>::K;
    constexpr int sb = kind_consts<KIND>::slot_bytes;
    if constexpr (AOS)
    {
        return *reinterpret_cast<const K*>(static_cast<const char*>(in0) + i * sb);
    }
    else
    {
        return reinterpret_cast<const K*>(in0)[i];
    }
}

template <int KIND>
SG_D uint32_t
part_of(typename kind_consts<KIND>::K key, int bits, int shift)
{
    return static_cast<uint32_t>(fibonacci_bucket(static_cast<uint64_t>(key), bits)) >> shift;
}

template <int KIND>
struct slot_image
{
    using type = typename std::conditional<kind_consts<KIND>::slot_bytes == 16, uint4,
                                           typename std::conditional<kind_consts<KIND>::slot_bytes == 8, uint2,
                                                                     unsigned int>::type>::type;
};

// A partitioned element of a table whose buckets come from caller-supplied hashes: the element's bytes and
// its key's hash, so the ordered kernels need not read the hash array at random positions.
template <typename E>
struct with_hash
{
    E e;
    uint64_t h;
};

// value_type bytes of (key, mapped); padding bytes are zero.
template <int KIND>
SG_D typename slot_image<KIND>::type
pack_element(typename kind_consts<KIND>::K key, typename kind_consts<KIND>::V val)
{
    using K = typename kind_consts<KIND>::K;
    using V = typename kind_consts<KIND>::V;
    uint32_t w[4] = { 0u, 0u, 0u, 0u };
    w[0] = static_cast<uint32_t>(key);
    if constexpr (sizeof(K) == 8)
    {
        w[1] = static_cast<uint32_t>(static_cast<uint64_t>(key) >> 32);
    }
    if constexpr (kind_traits<KIND>::is_map)
    {
        constexpr int vo = kind_traits<KIND>::val_offset / 4;
        w[vo] = static_cast<uint32_t>(val);
        if constexpr (sizeof(V) == 8)
        {
            w[vo + 1] = static_cast<uint32_t>(static_cast<uint64_t>(val) >> 32);
        }
    }
    constexpr int sb = kind_consts<KIND>::slot_bytes;
    if constexpr (sb == 16)
    {
        return make_uint4(w[0], w[1], w[2], w[3]);
    }
    else if constexpr (sb == 8)
    {
        return make_uint2(w[0], w[1]);
    }
    else
    {
        return w[0];
    }
}

// Scratch layout of a partitioned call: partition p owns elements [p * cap, (p + 1) * cap); elements past
// a partition's capacity go to the overflow region [parts * cap, parts * cap + ocap); an element that finds
// no room there either is not stored and sets *lost, and the direct kernel then runs over the whole input
// (inserting or erasing what is already in or out again changes nothing).  cap and ocap are multiples of
// the ordered kernel's chunk, so a chunk never straddles two regions.
struct part_layout
{
    int parts;
    int shift;          // part = bucket >> shift
    unsigned int cap;   // elements per partition
    unsigned int ocap;  // elements of the overflow region
    unsigned int* fill; // [kPartMax] elements offered to each partition (may exceed cap)
    unsigned int* ofill; // elements offered to the overflow region (may exceed ocap)
    unsigned int* lost;  // set when an element found no room
};

// One pass over the input: each block takes PER x kThreads elements, ranks them per partition in
// shared memory, reserves one range per partition (and one in the overflow region for what a partition
// has no room for), sorts the elements by partition in shared memory and writes each partition's run with
// consecutive threads, so stores reach L2 as whole lines rather than one request per element (random small
// writes cost as many requests as random line reads).
template <int KIND, bool AOS, int PER, bool HASHED = false>
__global__ void __launch_bounds__(kThreads, 6)
k_part_scatter(const void* in0, const void* in1, int64_t n, int bits, part_layout pl, void* out,
               const uint64_t* hashes = nullptr)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    using E = typename std::conditional<HASHED, with_hash<typename slot_image<KIND>::type>,
                                        typename slot_image<KIND>::type>::type;
    constexpr int kTileElems = PER * kThreads;
    __shared__ E stage[kTileElems];
    __shared__ uint8_t spid[kTileElems];
    __shared__ unsigned int cnt[kPartMax];
    __shared__ unsigned int loff[kPartMax];
    __shared__ unsigned int base[kPartMax];
    __shared__ unsigned int obase[kPartMax];
    E* dst = static_cast<E*>(out);
    const int lane = threadIdx.x & 31;
    for (int64_t tile = static_cast<int64_t>(blockIdx.x) * kTileElems; tile < n;
         tile += static_cast<int64_t>(gridDim.x) * kTileElems)
    {
        for (int p = threadIdx.x; p < kPartMax; p += blockDim.x)
        {
            cnt[p] = 0u;
        }
        __syncthreads();
        E elem[PER];
        uint32_t pid[PER];
        uint32_t rank[PER];
#pragma unroll
        for (int j = 0; j < PER; ++j)
        {
            const int64_t i = tile + j * kThreads + threadIdx.x;
            pid[j] = 0u;
            rank[j] = 0u;
            if (i < n)
            {
                K key;
                V val;
                load_input<KIND, AOS>(in0, in1, i, key, val);
                if constexpr (HASHED)
                {
                    const uint64_t h = __ldcs(hashes + i);
                    elem[j] = E{ pack_element<KIND>(key, val), h };
                    pid[j] = static_cast<uint32_t>(fibonacci_bucket(h, bits)) >> pl.shift;
                }
                else
                {
                    elem[j] = pack_element<KIND>(key, val);
                    pid[j] = part_of<KIND>(key, bits, pl.shift);
                }
                rank[j] = atomicAdd(&cnt[pid[j]], 1u);
            }
        }
        __syncthreads();
        if (threadIdx.x < 32)
        {
            // exclusive scan of cnt[0, kPartMax): lane l sums entries [8l, 8l + 8)
            constexpr int kPerLane = kPartMax / 32;
            unsigned int local = 0u;
#pragma unroll
            for (int k = 0; k < kPerLane; ++k)
            {
                local += cnt[lane * kPerLane + k];
            }
            unsigned int incl = local;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1)
            {
                const unsigned int x = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d)
                {
                    incl += x;
                }
            }
            unsigned int run = incl - local;
#pragma unroll
            for (int k = 0; k < kPerLane; ++k)
            {
                loff[lane * kPerLane + k] = run;
                run += cnt[lane * kPerLane + k];
            }
        }
        for (int p = threadIdx.x; p < pl.parts; p += blockDim.x)
        {
            const unsigned int c = cnt[p];
            unsigned int b = 0u;
            unsigned int ob = 0u;
            if (c != 0u)
            {
                b = atomicAdd(&pl.fill[p], c);
                const unsigned int room = b < pl.cap ? pl.cap - b : 0u;
                if (c > room)
                {
                    ob = atomicAdd(pl.ofill, c - room);
                }
            }
            base[p] = b;
            obase[p] = ob;
        }
        __syncthreads();
#pragma unroll
        for (int j = 0; j < PER; ++j)
        {
            const int64_t i = tile + j * kThreads + threadIdx.x;
            if (i < n)
            {
                const unsigned int pos = loff[pid[j]] + rank[j];
                stage[pos] = elem[j];
                spid[pos] = static_cast<uint8_t>(pid[j]);
            }
        }
        __syncthreads();
        const int count = n - tile < kTileElems ? static_cast<int>(n - tile) : kTileElems;
        for (int e = threadIdx.x; e < count; e += kThreads)
        {
            const unsigned int p = spid[e];
            const unsigned int r = static_cast<unsigned int>(e) - loff[p];
            const unsigned int b = base[p];
            const unsigned int room = b < pl.cap ? pl.cap - b : 0u;
            if (r < room)
            {
                dst[static_cast<int64_t>(p) * pl.cap + b + r] = stage[e];
            }
            else
            {
                const unsigned int o = obase[p] + (r - room);
                if (o < pl.ocap)
                {
                    dst[static_cast<int64_t>(pl.parts) * pl.cap + o] = stage[e];
                }
                else
                {
                    *pl.lost = 1u;
                }
            }
        }
        __syncthreads(); // the counters and the stage are rewritten by the next tile
    }
}

// Bulk insert over partitioned elements.  Blocks take chunks of kOrderedChunk elements in input order from
// a shared counter instead of a fixed stride, so no block drifts ahead: the elements in flight stay
// within about one partition, whose groups then stay in L2 while its keys arrive.
#ifndef SG_ORDERED_ITERS
#define SG_ORDERED_ITERS 16
#endif
constexpr int kOrderedChunk = SG_ORDERED_ITERS * kThreads;
// erase prefers short chunks (measured: 512 keys 1.26 ms, 4096 keys 1.48 ms for 2^25 keys)
#ifndef SG_ERASE_ORDERED_ITERS
#define SG_ERASE_ORDERED_ITERS 2
#endif
constexpr int kEraseChunk = SG_ERASE_ORDERED_ITERS * kThreads;

// Elements [first, last) of ordered chunk c of a partitioned scratch array: the chunks of partition 0, then
// of partition 1, ..., then of the overflow region; a chunk past its partition's fill is empty.  False once
// c is past the last element.
template <int CHUNK>
SG_D bool
ordered_chunk(const part_layout& pl, unsigned long long c, int64_t& first, int64_t& last)
{
    const unsigned long long per = pl.cap / CHUNK;
    const unsigned long long in_parts = per * static_cast<unsigned long long>(pl.parts);
    int64_t origin;
    unsigned long long off;
    unsigned int fill;
    if (c < in_parts)
    {
        const unsigned long long p = c / per;
        off = (c - p * per) * CHUNK;
        origin = static_cast<int64_t>(p) * pl.cap;
        fill = min(pl.fill[p], pl.cap);
    }
    else
    {
        // the overflow region is the last: its first empty chunk ends the walk
        off = (c - in_parts) * CHUNK;
        origin = static_cast<int64_t>(pl.parts) * pl.cap;
        fill = min(*pl.ofill, pl.ocap);
        if (off >= fill)
        {
            return false;
        }
    }
    first = origin + static_cast<int64_t>(off);
    last = off >= fill ? first : origin + static_cast<int64_t>(min(off + CHUNK, static_cast<unsigned long long>(fill)));
    return true;
}

// L2 prefetch ahead of the ordered insert.  Chunk (p, j) -- the j-th of the `per` chunks of partition p --
// is mapped onto the j-th of `per` equal slices of partition p's home-group range, so the claims, which run
// through the chunks in order, sweep the slot array front to back.  The block that claims chunk c issues a
// bulk L2 prefetch (cp.async.bulk.prefetch.L2, the TMA unit's L2 fill) of chunk c + SG_ORDERED_PREFETCH's
// slice: partitions ahead of the claim front arrive in L2 as sequential lines instead of each insert's
// random line read, and the dirty lines leave L2 in about the same order.  0 turns it off.
#ifndef SG_ORDERED_PREFETCH
#define SG_ORDERED_PREFETCH 0
#endif

SG_D void
prefetch_l2_bulk(const char* p, uint32_t bytes)
{
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Warp 0 of the calling block prefetches slice j of partition p's groups (p < parts); every address lies in
// the slot array, and every piece starts on a group boundary and is a whole number of groups.
template <int CHUNK>
SG_D void
prefetch_chunk_slice(const dview& t, const part_layout& pl, unsigned long long c)
{
    const unsigned long long per = pl.cap / CHUNK;
    const unsigned long long p = c / per;
    if (p >= static_cast<unsigned long long>(pl.parts))
    {
        return;
    }
    const unsigned long long j = c - p * per;
    const unsigned long long b_lo = p << pl.shift;
    const unsigned long long b_hi = (p + 1) << pl.shift;
    const unsigned long long g_lo = (b_lo * t.num_groups) >> t.bits;
    const unsigned long long g_hi = (b_hi * t.num_groups) >> t.bits;
    const unsigned long long ng = g_hi - g_lo;
    const unsigned long long s_lo = g_lo + ng * j / per;
    const unsigned long long s_hi = g_lo + ng * (j + 1) / per;
    const unsigned long long span = s_hi - s_lo; // groups of the slice
    const int lane = threadIdx.x & 31;
    const unsigned long long a = s_lo + span * lane / 32;
    const unsigned long long b = s_lo + span * (lane + 1) / 32;
    if (b > a && b <= t.num_groups)
    {
        prefetch_l2_bulk(t.slots + (a << 7), static_cast<uint32_t>((b - a) << 7));
    }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads, SG_ORDERED_MIN_BLOCKS)
k_insert_ordered(dview t, const void* in0, part_layout pl, unsigned long long* next_chunk)
{
    __shared__ unsigned long long s_claim;
    const tile_lanes L;
    const int warp = threadIdx.x >> 5;
    step_counts c;
    // thread 0 claims the block's next chunk while the current one is processed, so the claim's round
    // trip is hidden
    unsigned long long claimed = 0;
    if (threadIdx.x == 0)
    {
        claimed = atomicAdd(next_chunk, 1ull);
    }
    while (true)
    {
        if (threadIdx.x == 0)
        {
            s_claim = claimed;
        }
        __syncthreads();
        int64_t first, last;
        const unsigned long long cur = s_claim;
        const bool more = ordered_chunk<kOrderedChunk>(pl, cur, first, last);
        __syncthreads();
        if (!more)
        {
            break;
        }
        if (threadIdx.x == 0)
        {
            claimed = atomicAdd(next_chunk, 1ull);
        }
#if SG_ORDERED_PREFETCH > 0
        if (warp == 0)
        {
            prefetch_chunk_slice<kOrderedChunk>(t, pl, cur + SG_ORDERED_PREFETCH);
        }
#else
        (void)cur;
#endif
        for (int64_t base = first + warp * 32; base < last; base += kThreads)
        {
            const int64_t i = base + L.lane;
            insert_step<KIND, true>(t, L, in0, nullptr, i, i < last, nullptr, c);
        }
    }
    if (c.retry != 0)
    {
        atomicOr(&t.hdr->error, kErrRetry);
    }
    unsigned long long v[3] = { c.done, c.refused, 0ull - c.reused };
    unsigned long long* const dst[3] = { &t.hdr->size, &t.hdr->refused, &t.hdr->tombstones };
    block_add<3>(v, dst);
}

// Bulk erase over partitioned keys, chunks taken in order as in k_insert_ordered.
template <int KIND>
__global__ void __launch_bounds__(kThreads, SG_ORDERED_MIN_BLOCKS)
k_erase_ordered(dview t, const void* keys, part_layout pl, unsigned long long* next_chunk)
{
    __shared__ unsigned long long s_claim;
    const tile_lanes L;
    const int warp = threadIdx.x >> 5;
    step_counts c;
    // thread 0 claims the block's next chunk while the current one is processed, so the claim's round
    // trip is hidden
    unsigned long long claimed = 0;
    if (threadIdx.x == 0)
    {
        claimed = atomicAdd(next_chunk, 1ull);
    }
    while (true)
    {
        if (threadIdx.x == 0)
        {
            s_claim = claimed;
        }
        __syncthreads();
        int64_t first, last;
        const bool more = ordered_chunk<kEraseChunk>(pl, s_claim, first, last);
        __syncthreads();
        if (!more)
        {
            break;
        }
        if (threadIdx.x == 0)
        {
            claimed = atomicAdd(next_chunk, 1ull);
        }
        for (int64_t base = first + warp * 32; base < last; base += kThreads)
        {
            const int64_t i = base + L.lane;
            erase_step<KIND>(t, L, keys, i, i < last, nullptr, c);
        }
    }
    unsigned long long v[2] = { 0ull - c.done, c.done - c.oob };
    unsigned long long* const dst[2] = { &t.hdr->size, &t.hdr->tombstones };
    block_add<2>(v, dst);
}

// Ordered insert / erase with the input staged in shared memory.  The block's chunks are copied from the
// partitioned scratch array into a double buffer by bulk copies (cp.async.bulk, completed on an mbarrier):
// thread 0 stages chunk k + 1 while the warps probe chunk k, so every warp finds its 32 elements in shared
// memory when it reaches them and issues its home-group loads without first waiting for the input.
#ifndef SG_ORDERED_STAGE
#define SG_ORDERED_STAGE 1
#endif
#ifndef SG_STAGE_ITERS
#define SG_STAGE_ITERS 4
#endif
// ordered erase: consume each compare-and-swap one warp step later (erase_key_step_deferred)
#ifndef SG_ERASE_DEFER
#define SG_ERASE_DEFER 0
#endif
constexpr int kStageChunk = SG_STAGE_ITERS * kThreads;

template <int KIND, bool ERASE>
struct staged_elem
{
    using type = typename std::conditional<ERASE, typename kind_consts<KIND>::K, typename slot_image<KIND>::type>::type;
};

// The set kind holding the key type of KIND (erase partitions bare keys).
template <int KIND>
constexpr int keys_kind = sizeof(typename kind_consts<KIND>::K) == 8 ? SG_SET_U64 : SG_SET_U32;

// key / mapped value of a value_type image (padding ignored)
template <int KIND>
SG_D void
unpack_element(const typename slot_image<KIND>::type& e, typename kind_consts<KIND>::K& key,
               typename kind_consts<KIND>::V& val)
{
    constexpr int sb = kind_consts<KIND>::slot_bytes;
    if constexpr (sb == 16)
    {
        key = key_in_lane<KIND>(e, 0);
        val = value_in_lane<KIND>(e, 0);
    }
    else if constexpr (sb == 8)
    {
        const uint4 q = make_uint4(e.x, e.y, 0u, 0u);
        key = key_in_lane<KIND>(q, 0);
        val = value_in_lane<KIND>(q, 0);
    }
    else
    {
        key = static_cast<typename kind_consts<KIND>::K>(e);
        val = typename kind_consts<KIND>::V{};
    }
}

// resident blocks per SM the ordered erase is compiled for (its step holds fewer values than the insert's):
// 5 (48 registers) against 4 (64): 1.206 / 1.219 ms for the 2^25-key erase phase; 6 spills
#ifndef SG_ERASE_MIN_BLOCKS
#define SG_ERASE_MIN_BLOCKS 5
#endif
template <int KIND, bool ERASE, int CHUNK, bool HASHED = false>
__global__ void __launch_bounds__(kThreads, ERASE ? SG_ERASE_MIN_BLOCKS : SG_ORDERED_MIN_BLOCKS)
k_ordered_staged(dview t, const void* in, part_layout pl, unsigned long long* next_chunk)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    // with caller-supplied hashes the staged elements carry them (with_hash, written by k_part_scatter)
    using E = typename std::conditional<
            HASHED, with_hash<typename slot_image<ERASE ? keys_kind<KIND> : KIND>::type>,
            typename staged_elem<KIND, ERASE>::type>::type;
    static_assert(2 * CHUNK * sizeof(E) <= 40 * 1024, "staging buffers exceed the static shared memory budget");
    __shared__ __align__(128) E buf[2][CHUNK];
    __shared__ __align__(8) uint64_t full[2];
    __shared__ long long s_first[2];
    __shared__ long long s_last[2];
    const tile_lanes L;
    const int warp = threadIdx.x >> 5;
    const E* src = static_cast<const E*>(in);
    step_counts c;
    erase_pending<KIND> pend;

    // thread 0: chunk ch into buffer b.  Its range goes to s_first / s_last (s_first = -1 past the last chunk);
    // every call completes one phase of full[b], by the copy's bytes or, with nothing to copy, a plain arrival.
    // The copy is rounded up to 16 bytes; the rounded tail stays inside the chunk's region, whose capacity is
    // a whole number of chunks.
    auto stage = [&](unsigned long long ch, int b) {
        int64_t first, last;
        if (!ordered_chunk<CHUNK>(pl, ch, first, last))
        {
            first = last = -1;
        }
        s_first[b] = first;
        s_last[b] = last;
        if (last > first)
        {
            const uint32_t bytes = static_cast<uint32_t>(((last - first) * static_cast<int64_t>(sizeof(E)) + 15) & ~15ll);
            mbar_arrive_expect(&full[b], bytes);
            bulk_to_shared(&buf[b][0], src + first, bytes, &full[b]);
        }
        else
        {
            mbar_arrive(&full[b]);
        }
    };

    unsigned long long claimed = 0;
    if (threadIdx.x == 0)
    {
        mbar_init(&full[0], 1);
        mbar_init(&full[1], 1);
        fence_async_shared();
        stage(atomicAdd(next_chunk, 1ull), 0);
        claimed = atomicAdd(next_chunk, 1ull);
    }
    __syncthreads();
    for (int k = 0;; ++k)
    {
        const int b = k & 1;
        const long long first = s_first[b];
        const long long last = s_last[b];
        if (first < 0)
        {
            break;
        }
        if (threadIdx.x == 0)
        {
            // buffer b ^ 1 was released by the barrier that ended the previous chunk
            stage(claimed, b ^ 1);
            claimed = atomicAdd(next_chunk, 1ull);
        }
#if SG_ORDERED_PREFETCH > 0
        if (!ERASE && warp == 0)
        {
            // chunk index of this buffer: the block's claims are consecutive in `next_chunk` order only per
            // block, so the slice ahead is keyed on the chunk's own position
            const unsigned long long per = pl.cap / CHUNK;
            const unsigned long long cidx = static_cast<unsigned long long>(first / pl.cap) * per +
                                            static_cast<unsigned long long>(first % pl.cap) / CHUNK;
            if (first < static_cast<long long>(pl.parts) * pl.cap)
            {
                prefetch_chunk_slice<CHUNK>(t, pl, cidx + SG_ORDERED_PREFETCH);
            }
        }
#endif
        const bool ok = mbar_wait(&full[b], static_cast<uint32_t>(k >> 1) & 1u);
        if (__syncthreads_or(!ok))
        {
            if (threadIdx.x == 0)
            {
                atomicOr(&t.hdr->error, kErrStageWait);
                // the copy just staged into the other buffer, and a late one into this buffer
                mbar_wait(&full[b ^ 1], static_cast<uint32_t>((k + 1) >> 1) & 1u);
                mbar_wait(&full[b], static_cast<uint32_t>(k >> 1) & 1u);
            }
            break;
        }
        for (long long base = first + warp * 32; base < last; base += kThreads)
        {
            const long long i = base + L.lane;
            const bool valid = i < last;
            K key = C::empty_key;
            V val{};
            uint64_t h = 0;
            if (valid)
            {
                if constexpr (HASHED)
                {
                    const E& x = buf[b][i - first];
                    h = x.h;
                    if constexpr (ERASE)
                    {
                        typename kind_consts<keys_kind<KIND>>::K k2;
                        typename kind_consts<keys_kind<KIND>>::V v2;
                        unpack_element<keys_kind<KIND>>(x.e, k2, v2);
                        key = static_cast<K>(k2);
                    }
                    else
                    {
                        unpack_element<KIND>(x.e, key, val);
                    }
                }
                else if constexpr (ERASE)
                {
                    key = buf[b][i - first];
                }
                else
                {
                    unpack_element<KIND>(buf[b][i - first], key, val);
                }
            }
            if constexpr (HASHED)
            {
                if constexpr (ERASE)
                {
                    erase_key_step<KIND, true>(t, L, key, i, valid, nullptr, c, nullptr, h);
                }
                else
                {
                    insert_kv_step<KIND, true>(t, L, key, val, i, valid, nullptr, c, nullptr, h);
                }
            }
            else if constexpr (ERASE)
            {
#if SG_ERASE_DEFER
                erase_key_step_deferred<KIND>(t, L, key, valid, c, pend);
#else
                erase_key_step<KIND>(t, L, key, i, valid, nullptr, c);
#endif
            }
            else
            {
                insert_kv_step<KIND>(t, L, key, val, i, valid, nullptr, c);
            }
        }
        __syncthreads(); // buffer b is read; thread 0 may stage into it in the next iteration
    }
    if constexpr (ERASE)
    {
        c.done += erase_pending_done<KIND>(pend);
        unsigned long long v[2] = { 0ull - c.done, c.done - c.oob };
        unsigned long long* const dst[2] = { &t.hdr->size, &t.hdr->tombstones };
        block_add<2>(v, dst);
    }
    else
    {
        if (c.retry != 0)
        {
            atomicOr(&t.hdr->error, kErrRetry);
        }
        unsigned long long v[3] = { c.done, c.refused, 0ull - c.reused };
        unsigned long long* const dst[3] = { &t.hdr->size, &t.hdr->refused, &t.hdr->tombstones };
        block_add<3>(v, dst);
    }
}

// Bulk erase: src/stdgpu/impl/unordered_base_detail.cuh:1045-1066 (erase_from_key :497-522).
template <int KIND>
__global__ void __launch_bounds__(kThreads, SG_BULK_MIN_BLOCKS)
k_erase(dview t, const void* keys, int64_t n, uint8_t* out_flags, const uint64_t* hashes, const unsigned int* gate)
{
    if (gate != nullptr && *gate == 0u)
    {
        return;
    }
    const tile_lanes L;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    step_counts c;
    for (int64_t base = warp * 32; base < n; base += nwarps * 32)
    {
        const int64_t i = base + L.lane;
        erase_step<KIND>(t, L, keys, i, i < n, out_flags, c, hashes);
    }
    // size -= erased; tombstones += erased probed keys
    unsigned long long v[2] = { 0ull - c.done, c.done - c.oob };
    unsigned long long* const dst[2] = { &t.hdr->size, &t.hdr->tombstones };
    block_add<2>(v, dst);
}

// Bulk insert / erase of a table with the reference's excess-list accounting on: one thread per key through
// the device calls (sg::unordered_ref), which order the keys of one bucket under its stripe lock -- the
// reference's per-key path (insert_value / erase_from_key, unordered_base_detail.cuh:470-522).  The result
// is the reference's on one thread, which takes the keys in input order:
//  * k_counted_candidates first finds, per bucket, the smallest input index of a key not stored yet -- in
//    input order the first new key of that bucket, the one that takes the bucket's own slot if it is free;
//    every other new key takes an excess slot (and a later pass resets the candidates);
//  * a call of at most kCountedInOrderMax keys runs as one block, and when it could reach the refusal (the
//    excess list or the table could run out within it), one thread takes its keys in input order, so which
//    keys are refused is the same too.  A larger call that could reach it refuses keys in launch order.
constexpr int64_t kCountedInOrderMax = 4096;
constexpr uint32_t kNoCandidate = 0xFFFFFFFFu;

template <int KIND>
SG_D int64_t
counted_bucket(const sg_unordered_view& v, typename kind_consts<KIND>::K key, const uint64_t* hashes, int64_t i)
{
    const uint64_t h = hashes != nullptr ? __ldg(hashes + i) : identity_word_hash{}(key);
    return static_cast<int64_t>(fibonacci_bucket(h, v.bucket_bits));
}

// reset false: candidate per bucket (atomic minimum of the input indices of keys not stored); true: back to none.
template <int KIND, bool AOS>
__global__ void __launch_bounds__(kThreads)
k_counted_candidates(sg_unordered_view v, const void* in0, const void* in1, int64_t n, const uint64_t* hashes,
                     uint32_t* cand, bool reset)
{
    using C = kind_consts<KIND>;
    const sg::unordered_ref<KIND> ref{ v };
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    unsigned long long absent = 0, heads = 0;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        typename C::K key;
        typename C::V val;
        load_input<KIND, AOS>(in0, in1, i, key, val);
        const int64_t b = counted_bucket<KIND>(v, key, hashes, i);
        if (reset)
        {
            cand[b] = kNoCandidate;
        }
        else if (ref.find_slot_home(key, group_of_bucket(static_cast<uint64_t>(b), v.bucket_bits, v.num_groups)) < 0)
        {
            // bounds for k_insert_counted: keys not stored (copies counted each), buckets that get a first new
            // key while their own slot is free
            ++absent;
            if (atomicMin(cand + b, static_cast<uint32_t>(i)) == kNoCandidate && !bit_set(v.bucket_heads, b))
            {
                ++heads;
            }
        }
    }
    if (!reset)
    {
        unsigned long long c[2] = { absent, heads };
        unsigned long long* const dst[2] = { &ref.header()->count, &ref.header()->scratch };
        block_add<2>(c, dst);
    }
}

// The header counters' changes of a block's threads, added once.
SG_D void
flush_counts(table_header* h, const call_counts& c)
{
    unsigned long long v[4] = { static_cast<unsigned long long>(c.size), static_cast<unsigned long long>(c.tombs),
                                static_cast<unsigned long long>(c.refused), static_cast<unsigned long long>(c.excess) };
    unsigned long long* const dst[4] = { &h->size, &h->tombstones, &h->refused, &h->excess_used };
    block_add<4>(v, dst);
}

template <int KIND, bool AOS>
__global__ void __launch_bounds__(kThreads)
k_insert_counted(sg_unordered_view v, const void* in0, const void* in1, int64_t n, uint8_t* out_flags,
                 const uint64_t* hashes, const uint32_t* cand)
{
    using C = kind_consts<KIND>;
    sg::unordered_ref<KIND> ref{ v };
    // quiet: the call cannot reach the refusal -- it adds at most `absent` keys (k_counted_candidates), of which
    // at least `heads` take their buckets' own slots -- so it needs no lock and adds the counters at each
    // block's end (a block that starts after another block's flush sees larger counters and may take the
    // immediate path, which is always right)
    __shared__ int mode; // 0 quiet, 1 immediate, 2 in input order (one thread)
    if (threadIdx.x == 0)
    {
        const table_header* h = ref.header();
        const unsigned long long used = *reinterpret_cast<const volatile unsigned long long*>(&h->excess_used);
        const unsigned long long size = *reinterpret_cast<const volatile unsigned long long*>(&h->size);
        const unsigned long long absent = h->count, heads = h->scratch;
        const bool quiet = used + (absent - heads) < static_cast<unsigned long long>(v.excess_count) &&
                           size + absent < static_cast<unsigned long long>(v.total_count);
        mode = quiet ? 0 : (gridDim.x == 1 ? 2 : 1);
    }
    __syncthreads();
    int64_t first = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    call_counts counts;
    if (mode == 0)
    {
        ref.defer = &counts;
    }
    if (mode == 2)
    {
        if (threadIdx.x != 0)
        {
            return;
        }
        stride = 1;
    }
    for (int64_t i = first; i < n; i += stride)
    {
        typename C::K key;
        typename C::V val;
        load_input<KIND, AOS>(in0, in1, i, key, val);
        const int64_t b = counted_bucket<KIND>(v, key, hashes, i);
        // the bucket's own slot is for its candidate key (any copy of it)
        const uint32_t c = cand[b];
        bool first_new = false;
        if (c != kNoCandidate)
        {
            typename C::K ck;
            typename C::V cv;
            load_input<KIND, AOS>(in0, in1, static_cast<int64_t>(c), ck, cv);
            first_new = ck == key;
        }
        const int64_t slot = mode == 0 ? ref.insert_slot_quiet(key, val, b, first_new)
                                       : ref.insert_slot_bucket(key, val, b, first_new);
        if (out_flags != nullptr)
        {
            out_flags[i] = static_cast<uint8_t>(slot >= 0);
        }
    }
    if (mode == 0)
    {
        flush_counts(ref.header(), counts);
    }
}

template <int KIND>
__global__ void __launch_bounds__(kThreads)
k_erase_counted(sg_unordered_view v, const void* keys, int64_t n, uint8_t* out_flags, const uint64_t* hashes)
{
    using K = typename kind_consts<KIND>::K;
    // an erase-only launch: no lock (erase_quiet), and no insert reads the counters meanwhile, so they are
    // added at the block's end
    call_counts counts;
    sg::unordered_ref<KIND> ref{ v };
    ref.defer = &counts;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        const K key = __ldg(static_cast<const K*>(keys) + i);
        const int64_t r = hashes != nullptr ? ref.erase_quiet_hashed(key, __ldg(hashes + i))
                                            : ref.erase_quiet(key, ref.bucket(key));
        if (out_flags != nullptr)
        {
            out_flags[i] = static_cast<uint8_t>(r);
        }
    }
    flush_counts(ref.header(), counts);
}

// Bulk find / contains (device-only find/contains in the reference, :619-706).
template <int KIND, bool WANT_VALUES>
__global__ void __launch_bounds__(kThreads, SG_FIND_MIN_BLOCKS)
k_find(dview t, const void* keys, int64_t n, void* out_vals, uint8_t* out_found, const uint64_t* hashes)
{
    const tile_lanes L;
    const int64_t warp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (int64_t base = warp * 32; base < n; base += nwarps * 32)
    {
        const int64_t i = base + L.lane;
        find_step<KIND, WANT_VALUES>(t, L, keys, i, i < n, out_vals, out_found, hashes);
    }
}

// Bulk find / contains with the query keys staged in shared memory: each warp keeps a ring of
// SG_FIND_STAGES stages of its next 32 keys, filled by bulk copies that lane 0 issues SG_FIND_STAGES
// iterations ahead, so the home-group loads of an iteration start without waiting for its keys.  A
// partial last tile of 32 is loaded directly.  Keys must be 16-byte aligned (checked by the caller).
#ifndef SG_FIND_STAGE
#define SG_FIND_STAGE 0
#endif
#ifndef SG_FIND_STAGES
#define SG_FIND_STAGES 4
#endif

template <int KIND, bool WANT_VALUES>
__global__ void __launch_bounds__(kThreads, SG_FIND_MIN_BLOCKS)
k_find_staged(dview t, const void* keys, int64_t n, void* out_vals, uint8_t* out_found)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    constexpr int ST = SG_FIND_STAGES;
    constexpr int W = kThreads / 32;
    __shared__ __align__(128) K ring[W][ST][32];
    __shared__ __align__(8) uint64_t bars[W][ST];
    const tile_lanes L;
    const int w = threadIdx.x >> 5;
    const int64_t gwarp = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5;
    const K* src = static_cast<const K*>(keys);
    // lane 0: the 32 keys of iteration `it` into stage s -- a bulk copy when all 32 are in range, else a plain
    // arrival (the lanes then load their keys themselves); either completes one phase of bars[w][s]
    auto issue = [&](int64_t it, int st) {
        const int64_t base = (gwarp + it * nwarps) * 32;
        if (base + 32 <= n)
        {
            mbar_arrive_expect(&bars[w][st], 32 * sizeof(K));
            bulk_to_shared(&ring[w][st][0], src + base, 32 * sizeof(K), &bars[w][st]);
        }
        else
        {
            mbar_arrive(&bars[w][st]);
        }
    };
    if (L.lane == 0)
    {
        for (int st = 0; st < ST; ++st)
        {
            mbar_init(&bars[w][st], 1);
        }
        fence_async_shared();
        for (int st = 0; st < ST; ++st)
        {
            if ((gwarp + st * nwarps) * 32 < n)
            {
                issue(st, st);
            }
        }
    }
    __syncwarp();
    for (int64_t it = 0;; ++it)
    {
        const int64_t base = (gwarp + it * nwarps) * 32;
        if (base >= n)
        {
            break;
        }
        const int st = static_cast<int>(it % ST);
        const bool ok = mbar_wait(&bars[w][st], static_cast<uint32_t>(it / ST) & 1u);
        if (__any_sync(0xffffffffu, !ok))
        {
            if (L.lane == 0)
            {
                atomicOr(&t.hdr->error, kErrStageWait);
                for (int64_t j = it; j < it + ST; ++j) // copies still in flight, this one included
                {
                    if ((gwarp + j * nwarps) * 32 < n)
                    {
                        mbar_wait(&bars[w][j % ST], static_cast<uint32_t>(j / ST) & 1u);
                    }
                }
            }
            break;
        }
        const int64_t i = base + L.lane;
        const bool valid = i < n;
        K key = C::empty_key;
        if (valid)
        {
            key = base + 32 <= n ? ring[w][st][L.lane] : __ldcs(src + i);
        }
        __syncwarp();
        if (L.lane == 0 && (gwarp + (it + ST) * nwarps) * 32 < n)
        {
            fence_async_shared();
            issue(it + ST, st);
        }
        find_key_step<KIND, WANT_VALUES>(t, L, key, i, valid, out_vals, out_found);
    }
}

// valid(): every stored key is found at its own slot by its probe sequence, unused tail slots still hold
// the erased marker, and the stored-key count plus out-of-band keys equals size().
template <int KIND>
__global__ void __launch_bounds__(kThreads)
k_valid(dview t, sg_unordered_view v, unsigned long long* bad, bool check_reach)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    constexpr int G = C::slots_per_group;
    unordered_ref<KIND> ref{ v };
    const int64_t nslots = static_cast<int64_t>(t.num_groups) * G;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    unsigned long long live = 0, wrong = 0;
    for (int64_t s = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; s < nslots; s += stride)
    {
        const K k = __ldcg(reinterpret_cast<const K*>(t.slots + s * C::slot_bytes));
        if (s >= t.total)
        {
            wrong += (k != C::tomb_key);
            continue;
        }
        if (k == C::empty_key || k == C::tomb_key)
        {
            continue;
        }
        ++live;
        wrong += check_reach && (ref.find_slot(k) != s);
    }
    unsigned long long vv[2] = { live, wrong };
    unsigned long long* const dst[2] = { &t.hdr->count, bad };
    block_add<2>(vv, dst);
}

// valid() of the excess-list accounting: every set bit of slot_heads marks a stored key (and, with the
// table's own hash, one whose bucket's bit is set); hdr->count gets the number of such keys, `bad` the
// violations.
template <int KIND>
__global__ void __launch_bounds__(kThreads)
k_valid_heads(dview t, sg_unordered_view v, unsigned long long* bad, bool check_buckets)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    constexpr int G = C::slots_per_group;
    unordered_ref<KIND> ref{ v };
    const int64_t nslots = static_cast<int64_t>(t.num_groups) * G;
    const int64_t words = (nslots + 2 + 31) / 32;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    unsigned long long heads = 0, wrong = 0;
    for (int64_t w = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; w < words; w += stride)
    {
        unsigned bits = __ldcg(v.slot_heads + w);
        heads += static_cast<unsigned long long>(__popc(bits));
        while (bits != 0u)
        {
            const int64_t s = w * 32 + (__ffs(bits) - 1);
            bits &= bits - 1u;
            if (s >= nslots)
            {
                const int j = static_cast<int>(s - nslots);
                const K k = j == 0 ? C::empty_key : C::tomb_key;
                wrong += j > 1 || __ldcg(&t.hdr->special_state[j < 2 ? j : 0]) != 1u ||
                         (check_buckets && !bit_set(v.bucket_heads, ref.bucket(k)));
                continue;
            }
            const K k = __ldcg(reinterpret_cast<const K*>(t.slots + s * C::slot_bytes));
            wrong += s >= t.total || k == C::empty_key || k == C::tomb_key ||
                     (check_buckets && !bit_set(v.bucket_heads, ref.bucket(k)));
        }
    }
    unsigned long long vv[2] = { heads, wrong };
    unsigned long long* const dst[2] = { &t.hdr->count, bad };
    block_add<2>(vv, dst);
}

// Set bits of a word array into *out.
__global__ void __launch_bounds__(kThreads)
k_popc_words(const uint32_t* w, int64_t n, unsigned long long* out)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    unsigned long long c = 0;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        c += static_cast<unsigned long long>(__popc(__ldcg(w + i)));
    }
    unsigned long long vv[1] = { c };
    unsigned long long* const dst[1] = { out };
    block_add<1>(vv, dst);
}

// Compaction, pass 1: live slots per chunk of kRangeChunk slots.
template <int KIND>
__global__ void __launch_bounds__(kThreads)
k_range_count(dview t, unsigned int* chunk_counts)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    const int64_t c = blockIdx.x;
    const int64_t first = c * kRangeChunk;
    const int64_t limit = t.total;
    unsigned int live = 0;
#pragma unroll
    for (int r = 0; r < kRangeChunk / kThreads; ++r)
    {
        const int64_t s = first + r * kThreads + threadIdx.x;
        if (s < limit)
        {
            const K k = __ldcg(reinterpret_cast<const K*>(t.slots + s * C::slot_bytes));
            live += (k != C::empty_key && k != C::tomb_key);
        }
    }
    __shared__ unsigned int red[kThreads / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        live += __shfl_xor_sync(0xffffffffu, live, o);
    }
    if ((threadIdx.x & 31) == 0)
    {
        red[threadIdx.x >> 5] = live;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        unsigned int s = 0;
        for (int w = 0; w < kThreads / 32; ++w)
        {
            s += red[w];
        }
        chunk_counts[c] = s;
    }
}

// Compaction, pass 2: exclusive scan of the chunk counts (one block), then the out-of-band keys are
// appended after the probed ones; the total lands in hdr->count.
__global__ void __launch_bounds__(1024)
k_range_scan(unsigned int* chunk_counts, int64_t nchunks, table_header* hdr, int32_t* out_slots,
             int64_t special_base, int want_slots)
{
    __shared__ unsigned long long part[1024];
    const int64_t per = (nchunks + blockDim.x - 1) / blockDim.x;
    const int64_t lo = threadIdx.x * per;
    const int64_t hi = lo + per < nchunks ? lo + per : nchunks;
    unsigned long long s = 0;
    for (int64_t c = lo; c < hi; ++c)
    {
        s += chunk_counts[c];
    }
    part[threadIdx.x] = s;
    __syncthreads();
    if (threadIdx.x == 0)
    {
        unsigned long long run = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x); ++w)
        {
            const unsigned long long x = part[w];
            part[w] = run;
            run += x;
        }
        unsigned long long total = run;
        for (int sp = 0; sp < 2; ++sp)
        {
            if (hdr->special_state[sp] == 1u)
            {
                if (want_slots && out_slots != nullptr)
                {
                    out_slots[total] = static_cast<int32_t>(special_base + sp);
                }
                ++total;
            }
        }
        hdr->count = total;
    }
    __syncthreads();
    unsigned long long run = part[threadIdx.x];
    for (int64_t c = lo; c < hi; ++c)
    {
        const unsigned int x = chunk_counts[c];
        chunk_counts[c] = static_cast<unsigned int>(run);
        run += x;
    }
}

// Compaction, pass 3: write slot indices (or keys / mapped values) of live slots in slot order.
template <int KIND, bool SLOTS>
__global__ void __launch_bounds__(kThreads)
k_range_write(dview t, const unsigned int* chunk_offsets, int32_t* out_slots, void* out_keys, void* out_vals)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    const int64_t c = blockIdx.x;
    const int64_t first = c * kRangeChunk;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    __shared__ unsigned int warp_base[kThreads / 32];
    __shared__ unsigned int round_base;
    if (threadIdx.x == 0)
    {
        round_base = chunk_offsets[c];
    }
    __syncthreads();
    for (int r = 0; r < kRangeChunk / kThreads; ++r)
    {
        const int64_t s = first + r * kThreads + threadIdx.x;
        bool live = false;
        K k = C::empty_key;
        if (s < t.total)
        {
            k = __ldcg(reinterpret_cast<const K*>(t.slots + s * C::slot_bytes));
            live = (k != C::empty_key && k != C::tomb_key);
        }
        const unsigned b = __ballot_sync(0xffffffffu, live);
        if (lane == 0)
        {
            warp_base[warp] = __popc(b);
        }
        __syncthreads();
        unsigned int before = round_base;
        for (int w = 0; w < warp; ++w)
        {
            before += warp_base[w];
        }
        if (live)
        {
            const unsigned int pos = before + __popc(b & ((1u << lane) - 1u));
            if constexpr (SLOTS)
            {
                out_slots[pos] = static_cast<int32_t>(s);
            }
            else
            {
                if (out_keys != nullptr)
                {
                    reinterpret_cast<K*>(out_keys)[pos] = k;
                }
                if constexpr (kind_traits<KIND>::is_map)
                {
                    if (out_vals != nullptr)
                    {
                        reinterpret_cast<V*>(out_vals)[pos] = *reinterpret_cast<const V*>(
                                t.slots + s * C::slot_bytes + kind_traits<KIND>::val_offset);
                    }
                }
            }
        }
        __syncthreads();
        if (threadIdx.x == 0)
        {
            unsigned int add = 0;
            for (int w = 0; w < kThreads / 32; ++w)
            {
                add += warp_base[w];
            }
            round_base += add;
        }
        __syncthreads();
    }
}

// Appends the out-of-band keys (keys / mapped values) after the probed ones.
template <int KIND>
__global__ void
k_range_specials(dview t, const unsigned int* chunk_offsets, int64_t nchunks, const unsigned int* last_count,
                 void* out_keys, void* out_vals)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    unsigned long long pos = static_cast<unsigned long long>(chunk_offsets[nchunks - 1]) + *last_count;
    for (int sp = 0; sp < 2; ++sp)
    {
        if (t.hdr->special_state[sp] == 1u)
        {
            const int64_t slot = static_cast<int64_t>(t.num_groups) * C::slots_per_group + sp;
            if (out_keys != nullptr)
            {
                reinterpret_cast<K*>(out_keys)[pos] = sp == 0 ? C::empty_key : C::tomb_key;
            }
            if constexpr (kind_traits<KIND>::is_map)
            {
                if (out_vals != nullptr)
                {
                    reinterpret_cast<V*>(out_vals)[pos] =
                            *reinterpret_cast<const V*>(t.slots + slot * C::slot_bytes + kind_traits<KIND>::val_offset);
                }
            }
            ++pos;
        }
    }
}

} // namespace detail
} // namespace sg

// ====================================================================== host side

using namespace sg::detail;

// Pinned host mirrors of table headers, carved from 64 KB pinned pages that are kept for the process's
// life: a table's creation then costs no cudaMallocHost, which takes tens to hundreds of microseconds and
// serialises with other host-side CUDA calls.
class pinned_header_pool
{
public:
    void*
    get()
    {
        std::lock_guard<std::mutex> lock(m_);
        if (free_.empty())
        {
            void* page = nullptr;
            if (cudaMallocHost(&page, kPage) != cudaSuccess)
            {
                cudaGetLastError();
                return nullptr;
            }
            for (size_t off = 0; off + kPiece <= kPage; off += kPiece)
            {
                free_.push_back(static_cast<char*>(page) + off);
            }
        }
        void* p = free_.back();
        free_.pop_back();
        return p;
    }

    void
    put(void* p)
    {
        std::lock_guard<std::mutex> lock(m_);
        free_.push_back(p);
    }

private:
    static constexpr size_t kPage = size_t{ 64 } << 10;
    static constexpr size_t kPiece = (sizeof(sg::detail::table_header) + 63) / 64 * 64;
    std::mutex m_;
    std::vector<void*> free_;
};

inline pinned_header_pool&
pinned_headers()
{
    static pinned_header_pool* pool = new pinned_header_pool; // pages stay mapped until the process exits
    return *pool;
}

struct sg_unordered
{
    int32_t kind;
    int32_t slot_bytes;
    int64_t capacity;
    int64_t bucket_count;
    int64_t excess_count;
    int64_t total;
    int64_t num_groups;
    int bits;
    char* block;                // the one device block of slots, header, counters and locks
    char* slots;
    table_header* hdr;
    unsigned int* chunk_counts; // compaction scratch: one count per kRangeChunk slots, plus one
    int64_t nchunks;
    unsigned long long* host_hdr; // pinned mirror for synchronous reads
    int device;
    int32_t insert_mode;        // 0 automatic, 1 always direct, 2 partitioned whenever allowed
    bool custom_hash;           // buckets come from caller-supplied hashes (the *_hashed entry points)
    char* part_scratch;         // partitioned bulk insert: value_type elements, then 2 x kPartMax counters
    int64_t part_scratch_bytes;
    unsigned int* locks;        // stripe locks of the native device inserts (include/stdgpu_gb300/device.cuh)
    int64_t lock_count;
    object_allocator oa;           // the table's own allocator (sg_unordered_create_with_allocator), or none
    void (*release_ctx)(void* ctx); // called with oa.ctx when the table is destroyed (nullable)
    uint32_t* bucket_heads;        // the reference's excess-list accounting (sg_unordered_view), nullptr: off
    uint32_t* slot_heads;
    uint32_t* bucket_cand;         // a bulk insert's candidate per bucket (k_counted_candidates)
    char* heads_block;             // their own block when switched on after creation, else nullptr (in `block`)
    char* call_scratch;            // sg_unordered_call_scratch: the caller-side staging of the C++ API's bulk calls
    int64_t call_scratch_bytes;
};

namespace
{

bool
kind_ok(int32_t kind)
{
    return kind >= SG_SET_U32 && kind <= SG_MAP_U32_U64;
}

dview
view_of(const sg_unordered* t)
{
    return dview{ t->slots, t->hdr, static_cast<uint32_t>(t->num_groups), static_cast<uint32_t>(t->total), t->bits };
}

sg_unordered_view
public_view(const sg_unordered* t)
{
    sg_unordered_view v{};
    v.slots = t->slots;
    v.header = t->hdr;
    v.num_groups = t->num_groups;
    v.total_count = t->total;
    v.bucket_count = t->bucket_count;
    v.bucket_bits = t->bits;
    v.kind = t->kind;
    v.insert_locks = t->locks;
    v.lock_mask = t->lock_count - 1;
    v.bucket_heads = t->bucket_heads;
    v.slot_heads = t->slot_heads;
    v.excess_count = t->excess_count;
    return v;
}

// The excess-list accounting's two bit arrays: one bit per bucket, one per slot (the two out-of-band slots
// included), each rounded to 256 bytes.
#ifndef SG_ACCOUNTING_DEFAULT_MAX
#define SG_ACCOUNTING_DEFAULT_MAX (int64_t{ 1 } << 20) // on by default up to this max_size()
#endif
size_t
bucket_heads_bytes(int64_t bucket_count)
{
    return static_cast<size_t>((bucket_count + 2047) / 2048 * 256);
}

size_t
slot_heads_bytes(int64_t num_groups, int slot_bytes)
{
    const int64_t slots = num_groups * (kGroupBytes / slot_bytes) + 2;
    return static_cast<size_t>((slots + 2047) / 2048 * 256);
}

// a bulk insert's candidate per bucket (k_counted_candidates)
size_t
bucket_cand_bytes(int64_t bucket_count)
{
    return static_cast<size_t>((bucket_count * 4 + 255) / 256 * 256);
}

size_t
accounting_bytes(int64_t bucket_count, int64_t num_groups, int slot_bytes)
{
    return bucket_heads_bytes(bucket_count) + slot_heads_bytes(num_groups, slot_bytes) + bucket_cand_bytes(bucket_count);
}

// Stripe locks of the native device inserts: one per 16 probe groups, a power of two in [256, 2^22].
int64_t
insert_lock_count(int64_t num_groups)
{
    int64_t n = 256;
    while (n < num_groups / 16 && n < (int64_t{ 1 } << 22))
    {
        n <<= 1;
    }
    return n;
}

void
fill_geometry(int32_t kind, int64_t capacity, sg_geometry* g)
{
    int64_t b = 0, e = 0;
    reference_geometry(capacity, &b, &e);
    const int sb = slot_bytes_of_kind(kind);
    const int spg = kGroupBytes / sb;
    g->capacity = capacity;
    g->bucket_count = b;
    g->excess_count = e;
    g->max_size = b + e;
    g->num_groups = (g->max_size + spg - 1) / spg;
    g->slot_bytes = sb;
    g->slots_per_group = spg;
    const int64_t nchunks = (g->max_size + kRangeChunk - 1) / kRangeChunk;
    g->storage_bytes = (g->num_groups + 1) * kGroupBytes + static_cast<int64_t>(sizeof(table_header)) +
                       (nchunks + 1) * 4 + insert_lock_count(g->num_groups) * 4;
    if (g->max_size <= SG_ACCOUNTING_DEFAULT_MAX)
    {
        g->storage_bytes += static_cast<int64_t>(accounting_bytes(b, g->num_groups, sb));
    }
}

// Kernel dispatch over the six kinds.
template <template <int> class F, typename... Args>
sg_status
dispatch(int32_t kind, Args&&... args)
{
    switch (kind)
    {
        case 0:
            return F<0>::run(args...);
        case 1:
            return F<1>::run(args...);
        case 2:
            return F<2>::run(args...);
        case 3:
            return F<3>::run(args...);
        case 4:
            return F<4>::run(args...);
        case 5:
            return F<5>::run(args...);
        default:
            return SG_ERR_BAD_ARG;
    }
}

template <int KIND>
struct do_init
{
    static sg_status
    run(sg_unordered* t, cudaStream_t s)
    {
        static const int max_grid = persistent_grid(k_init<KIND>, kThreads);
        const int64_t units = (t->num_groups + 1) * (kGroupBytes / 16);
        k_init<KIND><<<grid_for(units, kThreads, max_grid), kThreads, 0, s>>>(view_of(t));
        SG_LAUNCH_CHECK();
        return SG_OK;
    }
};

// Partition count for a table: home-group ranges of about SG_PART_REGION_MB of slots.
#ifndef SG_PART_REGION_MB
#define SG_PART_REGION_MB 64
#endif
int
partitions_for(const sg_unordered* t)
{
    const int64_t bytes = (t->num_groups + 1) * kGroupBytes;
    int p = 2;
    while (p < kPartMax && static_cast<int64_t>(p) * (int64_t{ SG_PART_REGION_MB } << 20) < bytes)
    {
        p <<= 1;
    }
    return p <= (1 << t->bits) ? p : 0;
}

bool
use_partitioned_insert(const sg_unordered* t, int64_t n, const uint8_t* flags)
{
    if (flags != nullptr || n >= (int64_t{ 1 } << 31) || t->insert_mode == 1 || partitions_for(t) == 0)
    {
        return false;
    }
    if (t->insert_mode == 2)
    {
        return true;
    }
    const int64_t bytes = (t->num_groups + 1) * kGroupBytes;
    return n >= (int64_t{ 1 } << 22) && bytes >= (int64_t{ 256 } << 20) && n * 2 >= t->num_groups;
}

sg_status
ensure_part_scratch(sg_unordered* t, int64_t bytes)
{
    if (t->part_scratch_bytes >= bytes)
    {
        return SG_OK;
    }
    if (t->part_scratch != nullptr)
    {
        // a launch queued earlier may still read the old array
        SG_CUDA_TRY(cudaDeviceSynchronize());
        sg::detail::obj_free(t->oa, t->part_scratch);
        t->part_scratch = nullptr;
        t->part_scratch_bytes = 0;
    }
    const cudaError_t e = sg::detail::obj_malloc(t->oa, &t->part_scratch, static_cast<size_t>(bytes));
    if (e != cudaSuccess)
    {
        cudaGetLastError();
        t->part_scratch = nullptr;
        return e == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA;
    }
    t->part_scratch_bytes = bytes;
    if (reinterpret_cast<uintptr_t>(t->part_scratch) % 16 != 0)
    {
        // the staged kernels copy chunks of the array with 16-byte-aligned bulk copies; an allocator that
        // returned less alignment gets the direct kernels instead
        sg::detail::obj_free(t->oa, t->part_scratch);
        t->part_scratch = nullptr;
        t->part_scratch_bytes = 0;
        return SG_ERR_OOM;
    }
    return SG_OK;
}

// Partitions n input elements into the table's scratch array as PKIND's value_type elements (a set kind
// gives bare keys), in one pass: each partition gets room for its mean share plus 1/16 and two chunks, the
// overflow region n/16 plus one scatter tile.  Returns the layout and the ordered kernel's chunk counter,
// both zeroed.
template <int PKIND, bool AOS, int CHUNK, bool HASHED = false>
sg_status
partition_into_scratch(sg_unordered* t, const void* in0, const void* in1, int64_t n, cudaStream_t s, part_layout* pl,
                       unsigned long long** next_chunk, const uint64_t* hashes = nullptr)
{
    using E = typename std::conditional<HASHED, with_hash<typename slot_image<PKIND>::type>,
                                        typename slot_image<PKIND>::type>::type;
    const int parts = partitions_for(t);
    int shift = t->bits;
    for (int p = parts; p > 1; p >>= 1)
    {
        --shift;
    }
    const auto round_up = [](int64_t x, int64_t m) { return (x + m - 1) / m * m; };
    const int64_t mean = (n + parts - 1) / parts;
    const int64_t cap = round_up(mean + mean / 16 + 2 * CHUNK, CHUNK);
    constexpr int PER = part_per<PKIND>;
    const int64_t ocap = round_up(n / 16 + PER * kThreads, CHUNK);
    const int64_t ebytes = round_up((parts * cap + ocap) * static_cast<int64_t>(sizeof(E)), 256);
    constexpr int64_t kControlBytes = 2048; // fill[kPartMax], ofill, lost, then the 8-byte chunk counter
    sg_status st = ensure_part_scratch(t, ebytes + kControlBytes);
    if (st != SG_OK)
    {
        return st;
    }
    auto* control = reinterpret_cast<unsigned int*>(t->part_scratch + ebytes);
    SG_CUDA_TRY(cudaMemsetAsync(control, 0, kControlBytes, s));
    *pl = part_layout{ parts,   shift,          static_cast<unsigned int>(cap), static_cast<unsigned int>(ocap),
                       control, control + kPartMax, control + kPartMax + 1 };
    *next_chunk = reinterpret_cast<unsigned long long*>(control + kPartMax + 2);
    static const int g_scatter = persistent_grid(k_part_scatter<PKIND, AOS, PER, HASHED>, kThreads);
    k_part_scatter<PKIND, AOS, PER, HASHED><<<grid_for(n, kThreads * PER, g_scatter), kThreads, 0, s>>>(
            in0, in1, n, t->bits, *pl, t->part_scratch, hashes);
    SG_LAUNCH_CHECK();
    return SG_OK;
}

bool
use_partitioned_erase(const sg_unordered* t, int64_t n, const uint8_t* flags)
{
    if (flags != nullptr || n >= (int64_t{ 1 } << 31) || t->insert_mode == 1 || partitions_for(t) == 0)
    {
        return false;
    }
    if (t->insert_mode == 2)
    {
        return true;
    }
    const int64_t bytes = (t->num_groups + 1) * kGroupBytes;
    return n >= (int64_t{ 1 } << 22) && bytes >= (int64_t{ 256 } << 20);
}

// Bulk insert of a table with the accounting on: candidates, the inserts, candidates reset.
template <int KIND, bool AOS>
sg_status
insert_counted(sg_unordered* t, const void* in0, const void* in1, int64_t n, uint8_t* flags, cudaStream_t s,
               const uint64_t* hashes)
{
    if (n >= (int64_t{ 1 } << 32) - 1)
    {
        return SG_ERR_BAD_ARG; // candidates are 32-bit input indices
    }
    const sg_unordered_view v = public_view(t);
    static const int g_cand = persistent_grid(k_counted_candidates<KIND, AOS>, kThreads);
    static const int g_ins = persistent_grid(k_insert_counted<KIND, AOS>, kThreads);
    const int grid_cand = grid_for(n, kThreads, g_cand);
    SG_CUDA_TRY(cudaMemsetAsync(&t->hdr->count, 0, 2 * sizeof(unsigned long long), s));
    k_counted_candidates<KIND, AOS><<<grid_cand, kThreads, 0, s>>>(v, in0, in1, n, hashes, t->bucket_cand, false);
    SG_LAUNCH_CHECK();
    const int grid = n <= kCountedInOrderMax ? 1 : grid_for(n, kThreads, g_ins);
    k_insert_counted<KIND, AOS><<<grid, kThreads, 0, s>>>(v, in0, in1, n, flags, hashes, t->bucket_cand);
    SG_LAUNCH_CHECK();
    k_counted_candidates<KIND, AOS><<<grid_cand, kThreads, 0, s>>>(v, in0, in1, n, hashes, t->bucket_cand, true);
    SG_LAUNCH_CHECK();
    return SG_OK;
}

template <int KIND>
struct do_insert
{
    static sg_status
    run(sg_unordered* t, const void* in0, const void* in1, bool aos, int64_t n, uint8_t* flags, cudaStream_t s,
        const uint64_t* hashes = nullptr)
    {
        if (t->bucket_heads != nullptr)
        {
            return aos ? insert_counted<KIND, true>(t, in0, in1, n, flags, s, hashes)
                       : insert_counted<KIND, false>(t, in0, in1, n, flags, s, hashes);
        }
        part_layout pl{};
        unsigned long long* next_chunk = nullptr;
        sg_status st = SG_ERR_OOM;
        constexpr int kChunk = SG_ORDERED_STAGE ? kStageChunk : kOrderedChunk;
        constexpr int kChunkH = 512; // elements that carry their hash (with_hash): 32 bytes for 16-byte pairs
        if (use_partitioned_insert(t, n, flags) && (hashes == nullptr || SG_ORDERED_STAGE))
        {
            if (hashes == nullptr)
            {
                st = aos ? partition_into_scratch<KIND, true, kChunk>(t, in0, in1, n, s, &pl, &next_chunk)
                         : partition_into_scratch<KIND, false, kChunk>(t, in0, in1, n, s, &pl, &next_chunk);
            }
            else
            {
                st = aos ? partition_into_scratch<KIND, true, kChunkH, true>(t, in0, in1, n, s, &pl, &next_chunk, hashes)
                         : partition_into_scratch<KIND, false, kChunkH, true>(t, in0, in1, n, s, &pl, &next_chunk,
                                                                               hashes);
            }
            if (st != SG_OK && st != SG_ERR_OOM)
            {
                return st;
            }
        }
        // the direct kernel: without room for the scratch array it does the whole insert; after a partitioned
        // insert it is gated on the scatter having left elements out
        const unsigned int* gate = nullptr;
        if (st == SG_OK && hashes != nullptr)
        {
            if constexpr (SG_ORDERED_STAGE)
            {
                static const int max_grid = persistent_grid(k_ordered_staged<KIND, false, kChunkH, true>, kThreads);
                k_ordered_staged<KIND, false, kChunkH, true><<<grid_for(n, kChunkH, max_grid), kThreads, 0, s>>>(
                        view_of(t), t->part_scratch, pl, next_chunk);
            }
            SG_LAUNCH_CHECK();
            gate = pl.lost;
        }
        else if (st == SG_OK)
        {
            if constexpr (SG_ORDERED_STAGE)
            {
                static const int max_grid = persistent_grid(k_ordered_staged<KIND, false, kChunk>, kThreads);
                k_ordered_staged<KIND, false, kChunk><<<grid_for(n, kChunk, max_grid), kThreads, 0, s>>>(
                        view_of(t), t->part_scratch, pl, next_chunk);
            }
            else
            {
                static const int max_grid = persistent_grid(k_insert_ordered<KIND>, kThreads);
                k_insert_ordered<KIND><<<grid_for(n, kChunk, max_grid), kThreads, 0, s>>>(view_of(t),
                                                                                         t->part_scratch, pl,
                                                                                         next_chunk);
            }
            SG_LAUNCH_CHECK();
            gate = pl.lost;
        }
        if (aos)
        {
            static const int max_grid = persistent_grid(k_insert<KIND, true>, kThreads);
            k_insert<KIND, true><<<grid_for(n, kThreads, max_grid), kThreads, 0, s>>>(view_of(t), in0, in1, n, flags,
                                                                                     hashes, gate);
        }
        else
        {
            static const int max_grid = persistent_grid(k_insert<KIND, false>, kThreads);
            k_insert<KIND, false><<<grid_for(n, kThreads, max_grid), kThreads, 0, s>>>(view_of(t), in0, in1, n,
                                                                                      flags, hashes, gate);
        }
        SG_LAUNCH_CHECK();
        return SG_OK;
    }
};

template <int KIND>
struct do_erase
{
    static sg_status
    run(sg_unordered* t, const void* keys, int64_t n, uint8_t* flags, cudaStream_t s, const uint64_t* hashes = nullptr)
    {
        if (t->bucket_heads != nullptr)
        {
            static const int max_grid = persistent_grid(k_erase_counted<KIND>, kThreads);
            k_erase_counted<KIND><<<grid_for(n, kThreads, max_grid), kThreads, 0, s>>>(public_view(t), keys, n, flags,
                                                                                      hashes);
            SG_LAUNCH_CHECK();
            return SG_OK;
        }
        part_layout pl{};
        unsigned long long* next_chunk = nullptr;
        sg_status st = SG_ERR_OOM;
        if (use_partitioned_erase(t, n, flags) && (hashes == nullptr || SG_ORDERED_STAGE))
        {
            st = hashes == nullptr
                         ? partition_into_scratch<keys_kind<KIND>, false, kEraseChunk>(t, keys, nullptr, n, s, &pl,
                                                                                      &next_chunk)
                         : partition_into_scratch<keys_kind<KIND>, false, kEraseChunk, true>(t, keys, nullptr, n, s,
                                                                                            &pl, &next_chunk, hashes);
            if (st != SG_OK && st != SG_ERR_OOM)
            {
                return st;
            }
        }
        const unsigned int* gate = nullptr;
        if (st == SG_OK && hashes != nullptr)
        {
            if constexpr (SG_ORDERED_STAGE)
            {
                static const int g_ordered = persistent_grid(k_ordered_staged<KIND, true, kEraseChunk, true>, kThreads);
                k_ordered_staged<KIND, true, kEraseChunk, true><<<grid_for(n, kEraseChunk, g_ordered), kThreads, 0, s>>>(
                        view_of(t), t->part_scratch, pl, next_chunk);
            }
            SG_LAUNCH_CHECK();
            gate = pl.lost;
        }
        else if (st == SG_OK)
        {
            if constexpr (SG_ORDERED_STAGE)
            {
                static const int g_ordered = persistent_grid(k_ordered_staged<KIND, true, kEraseChunk>, kThreads);
                k_ordered_staged<KIND, true, kEraseChunk><<<grid_for(n, kEraseChunk, g_ordered), kThreads, 0, s>>>(
                        view_of(t), t->part_scratch, pl, next_chunk);
            }
            else
            {
                static const int g_ordered = persistent_grid(k_erase_ordered<KIND>, kThreads);
                k_erase_ordered<KIND><<<grid_for(n, kEraseChunk, g_ordered), kThreads, 0, s>>>(
                        view_of(t), t->part_scratch, pl, next_chunk);
            }
            SG_LAUNCH_CHECK();
            gate = pl.lost;
        }
        static const int max_grid = persistent_grid(k_erase<KIND>, kThreads);
        k_erase<KIND><<<grid_for(n, kThreads, max_grid), kThreads, 0, s>>>(view_of(t), keys, n, flags, hashes, gate);
        SG_LAUNCH_CHECK();
        return SG_OK;
    }
};

template <int KIND>
struct do_find
{
    static sg_status
    run(sg_unordered* t, const void* keys, int64_t n, void* vals, uint8_t* found, cudaStream_t s,
        const uint64_t* hashes = nullptr)
    {
        if (SG_FIND_STAGE && hashes == nullptr && reinterpret_cast<uintptr_t>(keys) % 16 == 0)
        {
            if (vals != nullptr)
            {
                static const int max_grid = persistent_grid(k_find_staged<KIND, true>, kThreads);
                k_find_staged<KIND, true><<<grid_for(n, kThreads, max_grid), kThreads, 0, s>>>(view_of(t), keys, n,
                                                                                              vals, found);
            }
            else
            {
                static const int max_grid = persistent_grid(k_find_staged<KIND, false>, kThreads);
                k_find_staged<KIND, false><<<grid_for(n, kThreads, max_grid), kThreads, 0, s>>>(view_of(t), keys, n,
                                                                                               vals, found);
            }
            SG_LAUNCH_CHECK();
            return SG_OK;
        }
        if (vals != nullptr)
        {
            static const int max_grid = persistent_grid(k_find<KIND, true>, kThreads);
            k_find<KIND, true><<<grid_for(n, kThreads, max_grid), kThreads, 0, s>>>(view_of(t), keys, n, vals, found,
                                                                                   hashes);
        }
        else
        {
            static const int max_grid = persistent_grid(k_find<KIND, false>, kThreads);
            k_find<KIND, false><<<grid_for(n, kThreads, max_grid), kThreads, 0, s>>>(view_of(t), keys, n, vals,
                                                                                    found, hashes);
        }
        SG_LAUNCH_CHECK();
        return SG_OK;
    }
};

template <int KIND>
struct do_valid
{
    static sg_status
    run(sg_unordered* t, unsigned long long* bad, cudaStream_t s)
    {
        static const int max_grid = persistent_grid(k_valid<KIND>, kThreads);
        const int64_t nslots = t->num_groups * (kGroupBytes / t->slot_bytes);
        k_valid<KIND><<<grid_for(nslots, kThreads, max_grid), kThreads, 0, s>>>(view_of(t), public_view(t), bad,
                                                                                !t->custom_hash);
        SG_LAUNCH_CHECK();
        return SG_OK;
    }
};

template <int KIND>
struct do_valid_heads
{
    static sg_status
    run(sg_unordered* t, unsigned long long* bad, cudaStream_t s)
    {
        static const int max_grid = persistent_grid(k_valid_heads<KIND>, kThreads);
        const int64_t words = (t->num_groups * (kGroupBytes / t->slot_bytes) + 2 + 31) / 32;
        k_valid_heads<KIND><<<grid_for(words, kThreads, max_grid), kThreads, 0, s>>>(view_of(t), public_view(t), bad,
                                                                                    !t->custom_hash);
        SG_LAUNCH_CHECK();
        return SG_OK;
    }
};

template <int KIND>
struct do_range
{
    static sg_status
    run(sg_unordered* t, int32_t* out_slots, void* out_keys, void* out_vals, cudaStream_t s)
    {
        const int64_t nch = t->nchunks;
        k_range_count<KIND><<<static_cast<unsigned>(nch), kThreads, 0, s>>>(view_of(t), t->chunk_counts);
        SG_LAUNCH_CHECK();
        // keep the last chunk's count for the tail append before the scan overwrites it
        SG_CUDA_TRY(cudaMemcpyAsync(t->chunk_counts + nch, t->chunk_counts + nch - 1, sizeof(unsigned int),
                                    cudaMemcpyDeviceToDevice, s));
        const int64_t special_base = t->num_groups * (kGroupBytes / t->slot_bytes);
        k_range_scan<<<1, 1024, 0, s>>>(t->chunk_counts, nch, t->hdr, out_slots, special_base, out_slots != nullptr);
        SG_LAUNCH_CHECK();
        if (out_slots != nullptr)
        {
            k_range_write<KIND, true><<<static_cast<unsigned>(nch), kThreads, 0, s>>>(view_of(t), t->chunk_counts,
                                                                                      out_slots, nullptr, nullptr);
            SG_LAUNCH_CHECK();
        }
        else
        {
            k_range_write<KIND, false><<<static_cast<unsigned>(nch), kThreads, 0, s>>>(view_of(t), t->chunk_counts,
                                                                                       nullptr, out_keys, out_vals);
            SG_LAUNCH_CHECK();
            k_range_specials<KIND><<<1, 1, 0, s>>>(view_of(t), t->chunk_counts, nch, t->chunk_counts + nch, out_keys,
                                                   out_vals);
            SG_LAUNCH_CHECK();
        }
        return SG_OK;
    }
};

sg_status
read_header(sg_unordered* t, cudaStream_t s)
{
    SG_CUDA_TRY(cudaMemcpyAsync(t->host_hdr, t->hdr, sizeof(table_header), cudaMemcpyDeviceToHost, s));
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    return SG_OK;
}

const table_header&
host_header(const sg_unordered* t)
{
    return *reinterpret_cast<const table_header*>(t->host_hdr);
}

} // namespace

namespace sg
{
namespace detail
{
void
unordered_accounting_off(sg_unordered* t)
{
    t->bucket_heads = nullptr;
    t->slot_heads = nullptr;
    t->bucket_cand = nullptr;
}
} // namespace detail
} // namespace sg

extern "C" {

sg_status
sg_set_device_allocator(sg_device_alloc_fn alloc, sg_device_free_fn release, void* ctx)
{
    if ((alloc == nullptr) != (release == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    device_allocator& a = allocator();
    if (a.live.load() != 0)
    {
        return SG_ERR_BAD_ARG;
    }
    a.alloc.store(alloc);
    a.release.store(release);
    a.ctx.store(ctx);
    return SG_OK;
}

int64_t
sg_live_device_allocations(void)
{
    return allocator().live.load();
}

sg_status
sg_unordered_geometry_for(int32_t kind, int64_t capacity, sg_geometry* out)
{
    if (!kind_ok(kind) || capacity <= 0 || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    fill_geometry(kind, capacity, out);
    if (out->max_size >= (int64_t{ 1 } << 31))
    {
        return SG_ERR_BAD_ARG;
    }
    return SG_OK;
}

namespace
{

// The accounting's arrays, carved from `base` (accounting_bytes of room).
void
place_accounting(sg_unordered* t, char* base)
{
    t->bucket_heads = reinterpret_cast<uint32_t*>(base);
    t->slot_heads = reinterpret_cast<uint32_t*>(base + bucket_heads_bytes(t->bucket_count));
    t->bucket_cand = reinterpret_cast<uint32_t*>(base + bucket_heads_bytes(t->bucket_count) +
                                                 slot_heads_bytes(t->num_groups, t->slot_bytes));
}

// The accounting of an empty table: no bucket's own slot taken, no excess slot used, no candidates.
sg_status
reset_accounting(sg_unordered* t, cudaStream_t s)
{
    if (t->bucket_heads == nullptr)
    {
        return SG_OK;
    }
    SG_CUDA_TRY(cudaMemsetAsync(t->bucket_heads, 0, bucket_heads_bytes(t->bucket_count), s));
    SG_CUDA_TRY(cudaMemsetAsync(t->slot_heads, 0, slot_heads_bytes(t->num_groups, t->slot_bytes), s));
    SG_CUDA_TRY(cudaMemsetAsync(t->bucket_cand, 0xFF, bucket_cand_bytes(t->bucket_count), s));
    SG_CUDA_TRY(cudaMemsetAsync(&t->hdr->excess_used, 0, sizeof(unsigned long long), s));
    return SG_OK;
}

sg_status
create_table(int32_t kind, int64_t capacity, const object_allocator& oa, void* stream, sg_unordered** out)
{
    if (out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    *out = nullptr;
    sg_geometry g{};
    sg_status st = sg_unordered_geometry_for(kind, capacity, &g);
    if (st != SG_OK)
    {
        return st;
    }
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess)
    {
        return SG_ERR_NO_DEVICE;
    }
    auto* t = new (std::nothrow) sg_unordered{};
    if (t == nullptr)
    {
        return SG_ERR_OOM;
    }
    t->kind = kind;
    t->slot_bytes = g.slot_bytes;
    t->capacity = capacity;
    t->bucket_count = g.bucket_count;
    t->excess_count = g.excess_count;
    t->total = g.max_size;
    t->num_groups = g.num_groups;
    t->bits = log2_exact(g.bucket_count);
    t->nchunks = (t->total + kRangeChunk - 1) / kRangeChunk;
    t->device = dev;
    t->oa = oa;
    // one device block: slots, then header, compaction counters and stripe locks at 256-byte offsets
    t->lock_count = insert_lock_count(t->num_groups);
    const auto up = [](size_t x) { return (x + 255) / 256 * 256; };
    const size_t off_hdr = up(static_cast<size_t>((t->num_groups + 1) * kGroupBytes));
    const size_t off_counts = off_hdr + up(sizeof(table_header));
    const size_t off_locks = off_counts + up(static_cast<size_t>(t->nchunks + 1) * sizeof(unsigned int));
    const bool accounting = t->total <= SG_ACCOUNTING_DEFAULT_MAX;
    const size_t off_bheads = off_locks + up(static_cast<size_t>(t->lock_count) * sizeof(unsigned int));
    const size_t block_bytes = accounting ? off_bheads + accounting_bytes(t->bucket_count, t->num_groups, t->slot_bytes)
                                          : off_locks + static_cast<size_t>(t->lock_count) * sizeof(unsigned int);
    cudaError_t e = sg::detail::obj_malloc(t->oa, &t->block, block_bytes);
    if (e == cudaSuccess)
    {
        t->slots = t->block;
        t->hdr = reinterpret_cast<table_header*>(t->block + off_hdr);
        t->chunk_counts = reinterpret_cast<unsigned int*>(t->block + off_counts);
        t->locks = reinterpret_cast<unsigned int*>(t->block + off_locks);
        if (accounting)
        {
            place_accounting(t, t->block + off_bheads);
        }
        t->host_hdr = static_cast<unsigned long long*>(pinned_headers().get());
        if (t->host_hdr == nullptr)
        {
            e = cudaErrorMemoryAllocation;
        }
    }
    if (e == cudaSuccess)
    {
        e = cudaMemsetAsync(t->locks, 0, static_cast<size_t>(t->lock_count) * sizeof(unsigned int), as_stream(stream));
    }
    if (e == cudaSuccess && accounting && reset_accounting(t, as_stream(stream)) != SG_OK)
    {
        e = cudaErrorUnknown;
    }
    if (e != cudaSuccess)
    {
        sg_unordered_destroy(t);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA;
    }
    st = dispatch<do_init>(kind, t, as_stream(stream));
    if (st != SG_OK)
    {
        sg_unordered_destroy(t);
        return st;
    }
    *out = t;
    return SG_OK;
}

// Switches the accounting of an empty table on or off (no checks); the arrays of a table created without
// them get their own block.
sg_status
set_accounting(sg_unordered* t, bool on, cudaStream_t s)
{
    if (!on)
    {
        t->bucket_heads = nullptr;
        t->slot_heads = nullptr;
        t->bucket_cand = nullptr;
        return SG_OK;
    }
    if (t->bucket_heads == nullptr)
    {
        const auto up = [](size_t x) { return (x + 255) / 256 * 256; };
        if (t->total <= SG_ACCOUNTING_DEFAULT_MAX)
        {
            // create_table placed them in the table's block, after the stripe locks
            const size_t off_counts = up(static_cast<size_t>((t->num_groups + 1) * kGroupBytes)) + up(sizeof(table_header));
            const size_t off_locks = off_counts + up(static_cast<size_t>(t->nchunks + 1) * sizeof(unsigned int));
            place_accounting(t, t->block + off_locks + up(static_cast<size_t>(t->lock_count) * sizeof(unsigned int)));
        }
        else
        {
            if (t->heads_block == nullptr &&
                sg::detail::obj_malloc(t->oa, &t->heads_block,
                                       accounting_bytes(t->bucket_count, t->num_groups, t->slot_bytes)) != cudaSuccess)
            {
                t->heads_block = nullptr;
                cudaGetLastError();
                return SG_ERR_OOM;
            }
            place_accounting(t, t->heads_block);
        }
    }
    return reset_accounting(t, s);
}

} // namespace

sg_status
sg_unordered_create(int32_t kind, int64_t capacity, void* stream, sg_unordered** out)
{
    return create_table(kind, capacity, object_allocator{}, stream, out);
}

sg_status
sg_unordered_create_with_allocator(int32_t kind, int64_t capacity, int32_t custom_hash, const sg_allocator* allocator,
                                   void* stream, sg_unordered** out)
{
    if (allocator == nullptr || allocator->alloc == nullptr || allocator->release == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    const sg_status st =
            create_table(kind, capacity, object_allocator{ allocator->alloc, allocator->release, allocator->ctx }, stream,
                         out);
    if (st != SG_OK)
    {
        return st;
    }
    (*out)->custom_hash = custom_hash != 0;
    (*out)->release_ctx = allocator->release_ctx;
    return SG_OK;
}

sg_status
sg_unordered_destroy(sg_unordered* t)
{
    if (t == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaError_t e = cudaSuccess;
    if (t->block != nullptr)
    {
        e = cudaDeviceSynchronize();
    }
    if (t->block != nullptr)
    {
        sg::detail::obj_free(t->oa, t->block);
    }
    if (t->part_scratch != nullptr)
    {
        sg::detail::obj_free(t->oa, t->part_scratch);
    }
    if (t->heads_block != nullptr)
    {
        sg::detail::obj_free(t->oa, t->heads_block);
    }
    if (t->call_scratch != nullptr)
    {
        sg::detail::obj_free(t->oa, t->call_scratch);
    }
    if (t->host_hdr != nullptr)
    {
        pinned_headers().put(t->host_hdr);
    }
    if (t->release_ctx != nullptr)
    {
        t->release_ctx(t->oa.ctx);
    }
    delete t;
    return e == cudaSuccess ? SG_OK : SG_ERR_CUDA;
}

sg_status
sg_unordered_insert(sg_unordered* t, const void* values, int64_t n, uint8_t* out_inserted, void* stream)
{
    if (t == nullptr || t->custom_hash || n < 0 || (n > 0 && values == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    return dispatch<do_insert>(t->kind, t, values, nullptr, true, n, out_inserted, as_stream(stream));
}

sg_status
sg_unordered_insert_kv(sg_unordered* t, const void* keys, const void* mapped, int64_t n, uint8_t* out_inserted,
                       void* stream)
{
    if (t == nullptr || t->custom_hash || n < 0 || (n > 0 && keys == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    return dispatch<do_insert>(t->kind, t, keys, mapped, false, n, out_inserted, as_stream(stream));
}

sg_status
sg_unordered_create_hashed(int32_t kind, int64_t capacity, void* stream, sg_unordered** out)
{
    const sg_status st = sg_unordered_create(kind, capacity, stream, out);
    if (st == SG_OK)
    {
        (*out)->custom_hash = true;
    }
    return st;
}

sg_status
sg_unordered_insert_hashed(sg_unordered* t, const void* keys, const void* mapped, const uint64_t* hashes, int64_t n,
                           uint8_t* out_inserted, void* stream)
{
    if (t == nullptr || !t->custom_hash || n < 0 || (n > 0 && (keys == nullptr || hashes == nullptr)))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    return dispatch<do_insert>(t->kind, t, keys, mapped, false, n, out_inserted, as_stream(stream), hashes);
}

sg_status
sg_unordered_erase_hashed(sg_unordered* t, const void* keys, const uint64_t* hashes, int64_t n, uint8_t* out_erased,
                          void* stream)
{
    if (t == nullptr || !t->custom_hash || n < 0 || (n > 0 && (keys == nullptr || hashes == nullptr)))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    return dispatch<do_erase>(t->kind, t, keys, n, out_erased, as_stream(stream), hashes);
}

sg_status
sg_unordered_find_hashed(sg_unordered* t, const void* keys, const uint64_t* hashes, int64_t n, void* out_mapped,
                         uint8_t* out_found, void* stream)
{
    if (t == nullptr || !t->custom_hash || n < 0 || (n > 0 && (keys == nullptr || hashes == nullptr)))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    const bool is_map = t->kind >= SG_MAP_U64_U32;
    return dispatch<do_find>(t->kind, t, keys, n, is_map ? out_mapped : nullptr, out_found, as_stream(stream), hashes);
}

sg_status
sg_unordered_contains_hashed(sg_unordered* t, const void* keys, const uint64_t* hashes, int64_t n,
                             uint8_t* out_flags, void* stream)
{
    if (t == nullptr || !t->custom_hash || n < 0 || (n > 0 && (keys == nullptr || hashes == nullptr)))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    return dispatch<do_find>(t->kind, t, keys, n, nullptr, out_flags, as_stream(stream), hashes);
}

sg_status
sg_unordered_is_hashed(const sg_unordered* t, int32_t* out)
{
    if (t == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    *out = t->custom_hash ? 1 : 0;
    return SG_OK;
}

sg_status
sg_unordered_rehash(sg_unordered* t, int64_t new_capacity, void* stream)
{
    if (t == nullptr || t->custom_hash)
    {
        return SG_ERR_BAD_ARG;
    }
    sg_geometry g{};
    sg_status st = sg_unordered_geometry_for(t->kind, new_capacity, &g);
    if (st != SG_OK)
    {
        return st;
    }
    cudaStream_t s = as_stream(stream);
    st = read_header(t, s);
    if (st != SG_OK)
    {
        return st;
    }
    const int64_t n = static_cast<int64_t>(host_header(t).size);
    const int kb = (t->kind == SG_SET_U32 || t->kind == SG_MAP_U32_U32 || t->kind == SG_MAP_U32_U64) ? 4 : 8;
    const int mb = t->kind == SG_MAP_U64_U32 || t->kind == SG_MAP_U32_U32 ? 4
                   : (t->kind == SG_MAP_U64_U64 || t->kind == SG_MAP_U32_U64) ? 8
                                                                             : 0;
    char* buf = nullptr;
    const int64_t cap = n + 2;
    const int64_t kbytes = ((cap * kb + 255) / 256) * 256;
    if (sg::detail::obj_malloc(t->oa, &buf, static_cast<size_t>(kbytes + cap * (mb > 0 ? mb : 1))) != cudaSuccess)
    {
        cudaGetLastError();
        return SG_ERR_OOM;
    }
    sg_unordered* fresh = nullptr;
    int64_t copied = 0;
    st = sg_unordered_range_copy(t, buf, mb > 0 ? buf + kbytes : nullptr, stream, &copied);
    if (st == SG_OK)
    {
        st = create_table(t->kind, new_capacity, t->oa, stream, &fresh);
    }
    if (st == SG_OK)
    {
        st = set_accounting(fresh, t->bucket_heads != nullptr, s);
    }
    if (st == SG_OK && copied > 0)
    {
        st = dispatch<do_insert>(fresh->kind, fresh, buf, mb > 0 ? buf + kbytes : nullptr, false, copied, nullptr, s);
    }
    int64_t refused = 0;
    if (st == SG_OK)
    {
        st = sg_unordered_status(fresh, stream, &refused, nullptr);
    }
    sg::detail::obj_free(t->oa, buf);
    if (st != SG_OK)
    {
        if (fresh != nullptr)
        {
            sg_unordered_destroy(fresh);
        }
        return st == SG_ERR_FULL ? SG_ERR_FULL : st;
    }
    // the table keeps its handle and its settings; the old storage leaves with `fresh`
    const int32_t mode = t->insert_mode;
    sg_unordered tmp = *t;
    *t = *fresh;
    *fresh = tmp;
    t->insert_mode = mode;
    t->release_ctx = tmp.release_ctx; // the handle keeps its allocator's context; the old storage leaves alone
    fresh->release_ctx = nullptr;
    return sg_unordered_destroy(fresh);
}

sg_status
sg_unordered_set_insert_mode(sg_unordered* t, int32_t mode)
{
    if (t == nullptr || mode < 0 || mode > 2)
    {
        return SG_ERR_BAD_ARG;
    }
    t->insert_mode = mode;
    return SG_OK;
}

sg_status
sg_unordered_erase(sg_unordered* t, const void* keys, int64_t n, uint8_t* out_erased, void* stream)
{
    if (t == nullptr || t->custom_hash || n < 0 || (n > 0 && keys == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    return dispatch<do_erase>(t->kind, t, keys, n, out_erased, as_stream(stream));
}

sg_status
sg_unordered_find(sg_unordered* t, const void* keys, int64_t n, void* out_mapped, uint8_t* out_found, void* stream)
{
    if (t == nullptr || t->custom_hash || n < 0 || (n > 0 && keys == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    const bool is_map = t->kind >= SG_MAP_U64_U32;
    return dispatch<do_find>(t->kind, t, keys, n, is_map ? out_mapped : nullptr, out_found, as_stream(stream));
}

sg_status
sg_unordered_contains(sg_unordered* t, const void* keys, int64_t n, uint8_t* out_flags, void* stream)
{
    if (t == nullptr || t->custom_hash || n < 0 || (n > 0 && (keys == nullptr || out_flags == nullptr)))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    return dispatch<do_find>(t->kind, t, keys, n, nullptr, out_flags, as_stream(stream));
}

sg_status
sg_unordered_size(sg_unordered* t, void* stream, int64_t* out_size)
{
    if (t == nullptr || out_size == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    sg_status st = read_header(t, as_stream(stream));
    if (st != SG_OK)
    {
        return st;
    }
    *out_size = static_cast<int64_t>(host_header(t).size);
    return (host_header(t).error & kErrRetry) != 0u ? SG_ERR_RETRY_EXHAUSTED : SG_OK;
}

sg_status
sg_unordered_status(sg_unordered* t, void* stream, int64_t* out_refused, int64_t* out_tombstones)
{
    if (t == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    sg_status st = read_header(t, as_stream(stream));
    if (st != SG_OK)
    {
        return st;
    }
    const table_header& h = host_header(t);
    if (out_refused != nullptr)
    {
        *out_refused = static_cast<int64_t>(h.refused);
    }
    if (out_tombstones != nullptr)
    {
        *out_tombstones = static_cast<int64_t>(h.tombstones);
    }
    if (h.refused != 0)
    {
        SG_CUDA_TRY(cudaMemsetAsync(&t->hdr->refused, 0, sizeof(unsigned long long), as_stream(stream)));
        return SG_ERR_FULL;
    }
    return (h.error & kErrRetry) != 0u ? SG_ERR_RETRY_EXHAUSTED : SG_OK;
}

sg_status
sg_unordered_clear(sg_unordered* t, void* stream)
{
    if (t == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    const sg_status st = reset_accounting(t, as_stream(stream));
    return st != SG_OK ? st : dispatch<do_init>(t->kind, t, as_stream(stream));
}

sg_status
sg_unordered_set_excess_accounting(sg_unordered* t, int32_t on, void* stream)
{
    if (t == nullptr || (on != 0 && on != 1))
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = as_stream(stream);
    sg_status st = read_header(t, s);
    if (st != SG_OK)
    {
        return st;
    }
    const table_header& h = host_header(t);
    if (h.size != 0)
    {
        return SG_ERR_BAD_ARG;
    }
    return set_accounting(t, on != 0, s);
}

sg_status
sg_unordered_call_scratch(sg_unordered* t, int64_t bytes, void* stream, void** out)
{
    if (t == nullptr || bytes < 0 || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    if (bytes > t->call_scratch_bytes)
    {
        if (t->call_scratch != nullptr)
        {
            // a call queued earlier may still read the old buffer
            SG_CUDA_TRY(cudaDeviceSynchronize());
            sg::detail::obj_free(t->oa, t->call_scratch);
            t->call_scratch = nullptr;
            t->call_scratch_bytes = 0;
        }
        const int64_t want = (bytes + (int64_t{ 1 } << 20) - 1) & ~((int64_t{ 1 } << 20) - 1);
        if (sg::detail::obj_malloc(t->oa, &t->call_scratch, static_cast<size_t>(want)) != cudaSuccess)
        {
            t->call_scratch = nullptr;
            cudaGetLastError();
            return SG_ERR_OOM;
        }
        t->call_scratch_bytes = want;
    }
    (void)stream;
    *out = t->call_scratch;
    return SG_OK;
}

sg_status
sg_unordered_excess_used(sg_unordered* t, void* stream, int64_t* out)
{
    if (t == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    if (t->bucket_heads == nullptr)
    {
        *out = -1;
        return SG_OK;
    }
    sg_status st = read_header(t, as_stream(stream));
    if (st != SG_OK)
    {
        return st;
    }
    *out = static_cast<int64_t>(host_header(t).excess_used);
    return SG_OK;
}

sg_status
sg_unordered_valid(sg_unordered* t, void* stream, int32_t* out_valid)
{
    if (t == nullptr || out_valid == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = as_stream(stream);
    // hdr->count accumulates live slots; hdr->scratch accumulates violations
    SG_CUDA_TRY(cudaMemsetAsync(&t->hdr->count, 0, 2 * sizeof(unsigned long long), s));
    sg_status st = dispatch<do_valid>(t->kind, t, &t->hdr->scratch, s);
    if (st != SG_OK)
    {
        return st;
    }
    st = read_header(t, s);
    if (st != SG_OK)
    {
        return st;
    }
    const table_header& h = host_header(t);
    unsigned long long specials = 0;
    bool ok = true;
    for (int sp = 0; sp < 2; ++sp)
    {
        ok = ok && (h.special_state[sp] <= 1u);
        specials += (h.special_state[sp] == 1u);
    }
    ok = ok && h.scratch == 0 && (h.count + specials == h.size);
    if (ok && t->bucket_heads != nullptr)
    {
        // the accounting: keys marked as holding their bucket's own slot, as many as buckets marked taken,
        // and with the keys in excess slots they make up the size
        const unsigned long long size = h.size, used = h.excess_used;
        SG_CUDA_TRY(cudaMemsetAsync(&t->hdr->count, 0, 2 * sizeof(unsigned long long), s));
        st = dispatch<do_valid_heads>(t->kind, t, &t->hdr->scratch, s);
        if (st == SG_OK)
        {
            st = read_header(t, s);
        }
        if (st != SG_OK)
        {
            return st;
        }
        const unsigned long long heads = h.count;
        ok = h.scratch == 0 && used <= static_cast<unsigned long long>(t->excess_count) && heads + used == size;
        SG_CUDA_TRY(cudaMemsetAsync(&t->hdr->count, 0, sizeof(unsigned long long), s));
        const int64_t words = (t->bucket_count + 31) / 32;
        static const int max_grid = persistent_grid(k_popc_words, kThreads);
        k_popc_words<<<grid_for(words, kThreads, max_grid), kThreads, 0, s>>>(t->bucket_heads, words, &t->hdr->count);
        SG_LAUNCH_CHECK();
        st = read_header(t, s);
        if (st != SG_OK)
        {
            return st;
        }
        ok = ok && h.count == heads;
    }
    *out_valid = ok ? 1 : 0;
    return SG_OK;
}

sg_status
sg_unordered_device_range(sg_unordered* t, int32_t* out_slots, void* stream, int64_t* out_n)
{
    if (t == nullptr || out_slots == nullptr || out_n == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = as_stream(stream);
    sg_status st = dispatch<do_range>(t->kind, t, out_slots, nullptr, nullptr, s);
    if (st != SG_OK)
    {
        return st;
    }
    st = read_header(t, s);
    if (st != SG_OK)
    {
        return st;
    }
    *out_n = static_cast<int64_t>(host_header(t).count);
    return SG_OK;
}

sg_status
sg_unordered_range_copy(sg_unordered* t, void* out_keys, void* out_mapped, void* stream, int64_t* out_n)
{
    if (t == nullptr || out_n == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = as_stream(stream);
    const bool is_map = t->kind >= SG_MAP_U64_U32;
    sg_status st = dispatch<do_range>(t->kind, t, nullptr, out_keys, is_map ? out_mapped : nullptr, s);
    if (st != SG_OK)
    {
        return st;
    }
    st = read_header(t, s);
    if (st != SG_OK)
    {
        return st;
    }
    *out_n = static_cast<int64_t>(host_header(t).count);
    return SG_OK;
}

sg_status
sg_unordered_bucket(const sg_unordered* t, const void* key, int64_t* out_bucket)
{
    if (t == nullptr || t->custom_hash || key == nullptr || out_bucket == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    uint64_t k = 0;
    if (t->kind == SG_SET_U32 || t->kind == SG_MAP_U32_U32 || t->kind == SG_MAP_U32_U64)
    {
        k = *static_cast<const uint32_t*>(key);
    }
    else
    {
        k = *static_cast<const uint64_t*>(key);
    }
    *out_bucket = static_cast<int64_t>(fibonacci_bucket(k, t->bits));
    return SG_OK;
}

sg_status
sg_unordered_bucket_of_hash(const sg_unordered* t, uint64_t hash, int64_t* out_bucket)
{
    if (t == nullptr || out_bucket == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    *out_bucket = static_cast<int64_t>(fibonacci_bucket(hash, t->bits));
    return SG_OK;
}

sg_status
sg_unordered_geometry(const sg_unordered* t, sg_geometry* out)
{
    if (t == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    fill_geometry(t->kind, t->capacity, out);
    return SG_OK;
}

sg_status
sg_unordered_view_of(const sg_unordered* t, sg_unordered_view* out)
{
    if (t == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    *out = public_view(t);
    return SG_OK;
}

int64_t
sg_kernel_launch_count(void)
{
    return g_launches.load(std::memory_order_relaxed);
}

const char*
sg_status_string(sg_status s)
{
    switch (s)
    {
        case SG_OK:
            return "ok";
        case SG_ERR_FULL:
            return "container full: elements were refused";
        case SG_ERR_BAD_ARG:
            return "bad argument";
        case SG_ERR_OOM:
            return "device allocation failed";
        case SG_ERR_BUDGET:
            return "refused by the memory budget";
        case SG_ERR_RETRY_EXHAUSTED:
            return "a bounded device wait or retry gave up";
        case SG_ERR_CUDA:
            return "CUDA runtime error";
        case SG_ERR_NO_DEVICE:
            return "no usable device";
        default:
            return "unknown status";
    }
}

} // extern "C"

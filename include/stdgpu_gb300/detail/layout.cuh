// Storage layout of the GB300 hash table, shared by the library kernels and by the
// native device API (include/stdgpu_gb300/device.cuh).
//
// Slots hold the reference's value_type byte for byte (Key for sets,
// stdgpu::pair<const Key, T> for maps; src/stdgpu/unordered_map.cuh:80,
// src/stdgpu/unordered_set.cuh:69), packed into 128-byte probe groups:
// 32 slots of 4 B, 16 of 8 B or 8 of 16 B.  A key's home group comes from the
// reference's own bucket(key) (fibonacci hashing of the identity hash,
// src/stdgpu/impl/unordered_base_detail.cuh:56-85, :547-564) scaled from
// bucket_count buckets onto num_groups groups, so keys that share a reference
// bucket share a home group.  Probing is linear over whole groups.
//
// The key word of a slot carries its state: all-ones = never used (EMPTY),
// all-ones minus one = erased (TOMB), anything else = a stored key.  Keys equal
// to those two values are stored out of band in the two slots of the extra
// group after the last probe group, with their presence in the device header,
// so every key value of the type is accepted, as in the reference.
//
// Slots at index >= total_count (the reference's max_size()) in the last probe
// group are set to TOMB at creation and never claimed, so a table holds at most
// max_size() probed keys, as the reference does.
#ifndef STDGPU_GB300_DETAIL_LAYOUT_CUH
#define STDGPU_GB300_DETAIL_LAYOUT_CUH

#include <stdint.h>

#if defined(__CUDACC__)
#define SG_HD __host__ __device__ __forceinline__
#define SG_D __device__ __forceinline__
#else
#define SG_HD inline
#define SG_D inline
#endif

namespace sg
{
namespace detail
{

constexpr int kGroupBytes = 128;
constexpr int kTileLanes = 8; // lanes cooperating on one probe group, 16 B each

// Device-resident counters of one table.
struct table_header
{
    unsigned long long size;       // stored elements, out-of-band keys included
    unsigned long long refused;    // inserts refused because no slot was free (reported, then reset)
    unsigned long long tombstones; // erased slots not yet reused
    unsigned int special_state[2]; // out-of-band keys EMPTY-valued [0] / TOMB-valued [1]: 0 absent, 1 present, 2 writing
    unsigned int error;            // sticky error bits (kErr*)
    unsigned int pad0;
    unsigned long long count;      // per-call scratch counter (valid / range)
    unsigned long long scratch;    // per-call scratch counter (valid: violations)
    unsigned long long excess_used; // keys holding one of the reference's excess slots (excess-list accounting)
};

// Changes to a table's header counters that a bulk kernel's thread accumulates and its block adds once.
struct call_counts
{
    long long size = 0;
    long long tombs = 0;
    long long refused = 0;
    long long excess = 0;
};

constexpr unsigned int kErrRetry = 1u;      // a CAS retry loop gave up
constexpr unsigned int kErrIndex = 2u;      // an index outside the table was computed (never expected)

// Kind traits: Key, mapped type and where they sit in a slot.
template <int KIND>
struct kind_traits;

struct no_value
{
};

template <>
struct kind_traits<0> // unordered_set<uint32_t>
{
    using key_type = uint32_t;
    using mapped_type = uint32_t; // unused
    static constexpr bool is_map = false;
    static constexpr int slot_bytes = 4;
    static constexpr int val_offset = 0;
};
template <>
struct kind_traits<1> // unordered_set<uint64_t>
{
    using key_type = uint64_t;
    using mapped_type = uint64_t; // unused
    static constexpr bool is_map = false;
    static constexpr int slot_bytes = 8;
    static constexpr int val_offset = 0;
};
template <>
struct kind_traits<2> // unordered_map<uint64_t, uint32_t>
{
    using key_type = uint64_t;
    using mapped_type = uint32_t;
    static constexpr bool is_map = true;
    static constexpr int slot_bytes = 16;
    static constexpr int val_offset = 8;
};
template <>
struct kind_traits<3> // unordered_map<uint64_t, uint64_t>
{
    using key_type = uint64_t;
    using mapped_type = uint64_t;
    static constexpr bool is_map = true;
    static constexpr int slot_bytes = 16;
    static constexpr int val_offset = 8;
};
template <>
struct kind_traits<4> // unordered_map<uint32_t, uint32_t>
{
    using key_type = uint32_t;
    using mapped_type = uint32_t;
    static constexpr bool is_map = true;
    static constexpr int slot_bytes = 8;
    static constexpr int val_offset = 4;
};
template <>
struct kind_traits<5> // unordered_map<uint32_t, uint64_t>
{
    using key_type = uint32_t;
    using mapped_type = uint64_t;
    static constexpr bool is_map = true;
    static constexpr int slot_bytes = 16;
    static constexpr int val_offset = 8;
};

template <int KIND>
struct kind_consts
{
    using K = typename kind_traits<KIND>::key_type;
    using V = typename kind_traits<KIND>::mapped_type;
    static constexpr int slot_bytes = kind_traits<KIND>::slot_bytes;
    static constexpr int slots_per_group = kGroupBytes / slot_bytes;
    static constexpr int slots_per_lane = 16 / slot_bytes; // slots in one lane's 16-byte share of a group
    static constexpr K empty_key = static_cast<K>(~static_cast<K>(0));
    static constexpr K tomb_key = static_cast<K>(~static_cast<K>(0) - 1);
};

SG_HD int slot_bytes_of_kind(int kind)
{
    return kind == 0 ? 4 : (kind == 1 || kind == 4) ? 8 : 16;
}

// fibonacci_hashing(hash, 2^bits): src/stdgpu/impl/unordered_base_detail.cuh:56-85
SG_HD uint64_t fibonacci_bucket(uint64_t hash, int bits)
{
    if (bits <= 0)
    {
        return 0;
    }
    const unsigned drop = 64u - static_cast<unsigned>(bits);
    const uint64_t improved = hash ^ (hash >> drop);
    return (improved * 11400714819323198485ull) >> drop;
}

// Home probe group of a reference bucket.
SG_HD int64_t group_of_bucket(uint64_t bucket, int bits, int64_t num_groups)
{
    return static_cast<int64_t>((bucket * static_cast<uint64_t>(num_groups)) >> bits);
}

SG_HD int64_t next_group(int64_t g, int64_t num_groups)
{
    return (g + 1 == num_groups) ? 0 : g + 1;
}

// Extract sub-slot s (0 .. slots_per_lane-1) of a lane's 16-byte share.
template <int KIND>
SG_HD typename kind_consts<KIND>::K key_in_lane(const uint4& d, int s)
{
    using K = typename kind_consts<KIND>::K;
    constexpr int sb = kind_consts<KIND>::slot_bytes;
    if constexpr (sb == 4)
    {
        return static_cast<K>(s == 0 ? d.x : s == 1 ? d.y : s == 2 ? d.z : d.w);
    }
    else if constexpr (sb == 8)
    {
        if constexpr (sizeof(K) == 8)
        {
            return s == 0 ? (static_cast<uint64_t>(d.y) << 32 | d.x) : (static_cast<uint64_t>(d.w) << 32 | d.z);
        }
        else
        {
            return static_cast<K>(s == 0 ? d.x : d.z);
        }
    }
    else
    {
        if constexpr (sizeof(K) == 8)
        {
            return static_cast<uint64_t>(d.y) << 32 | d.x;
        }
        else
        {
            return static_cast<K>(d.x);
        }
    }
}

template <int KIND>
SG_HD typename kind_consts<KIND>::V value_in_lane(const uint4& d, int s)
{
    using V = typename kind_consts<KIND>::V;
    constexpr int sb = kind_consts<KIND>::slot_bytes;
    if constexpr (!kind_traits<KIND>::is_map)
    {
        return V{};
    }
    else if constexpr (sb == 8) // pair<u32,u32>
    {
        return static_cast<V>(s == 0 ? d.y : d.w);
    }
    else // 16-byte pair, value at offset 8
    {
        if constexpr (sizeof(V) == 8)
        {
            return static_cast<uint64_t>(d.w) << 32 | d.z;
        }
        else
        {
            return static_cast<V>(d.z);
        }
    }
}

// The reference's hash<uint32_t> / hash<uint64_t> is the identity (src/stdgpu/impl/functional_detail.h:60-80):
// the bucket of an integer key is the fibonacci hashing of the key itself.
struct identity_word_hash
{
    template <typename K>
    SG_HD uint64_t
    operator()(K key_word) const
    {
        return static_cast<uint64_t>(key_word);
    }
};

#if defined(__CUDACC__)
// Acquire-release fence at device scope: a lock's acquire after the compare-and-swap that took it, its release
// before the store that frees it (lighter than __threadfence's sequentially consistent fence).
__device__ __forceinline__ void
fence_acq_rel_gpu()
{
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
}
#endif

// ---- deque ring state, shared by the library's bulk kernels and the device-side calls of
// stdgpu_gb300/stdgpu.cuh.  A deque of capacity c is a ring of c slots plus one 32-bit turn word per slot:
// push k and pop k use slot (ticket k) mod c; the k-th push waits for turn k, writes, and sets k + 1; the
// k-th pop waits for k + 1, reads, and sets k + c.  Tickets start at c x 2^32 (a multiple of c and of 2^32).
constexpr unsigned int kDequeErrWait = 1u;
constexpr long long kWaitLimit = 1ll << 22; // polls of a ring slot before giving up (about 1-2 s with backoff)

// size guards the capacity: a push reservation adds to it first, a pop reservation subtracts from it
// only after its tickets are claimed.  avail guards pop_front: a push reservation adds to it only after
// its tickets are claimed, a pop reservation subtracts from it first.  So a pop is only reserved for a
// ticket that a push has claimed, and a push only for a slot whose previous pop has been claimed; an
// over-reservation is undone and can make a concurrent reservation fail near the bounds, never succeed
// wrongly.  Both equal the element count when no launch is running.
struct deque_counters
{
    long long size;
    unsigned long long begin;
    unsigned long long end;
    unsigned int error;
    unsigned int pad;
    long long avail;
    unsigned long long op_t0; // push_front / pop_back launches: the end before the launch
    long long op_k;           // and how many elements it moves
};


#if defined(__CUDACC__)
SG_D bool
wait_turn(const unsigned* seq, unsigned want, unsigned* error)
{
    long long polls = 0;
    unsigned backoff = 32;
    while (true)
    {
        unsigned cur;
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(cur) : "l"(seq) : "memory");
        if (cur == want)
        {
            return true;
        }
        if (++polls > kWaitLimit)
        {
            atomicOr(error, kDequeErrWait);
            return false;
        }
        __nanosleep(backoff);
        backoff = backoff < 256 ? backoff * 2 : 256;
    }
}

SG_D void
store_turn(unsigned* seq, unsigned v)
{
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(seq), "r"(v) : "memory");
}


// 16-byte compare-and-swap (sm_90 and later): old <- *p; if old == expected then *p <- desired.
SG_D void
cas128(void* p, unsigned long long e_lo, unsigned long long e_hi, unsigned long long d_lo, unsigned long long d_hi,
       unsigned long long& o_lo, unsigned long long& o_hi)
{
    asm volatile("{\n\t.reg .b128 d, b, c;\n\t"
                 "mov.b128 b, {%2, %3};\n\t"
                 "mov.b128 c, {%4, %5};\n\t"
                 "atom.global.cas.b128 d, [%6], b, c;\n\t"
                 "mov.b128 {%0, %1}, d;\n\t}"
                 : "=l"(o_lo), "=l"(o_hi)
                 : "l"(e_lo), "l"(e_hi), "l"(d_lo), "l"(d_hi), "l"(p)
                 : "memory");
}

SG_D unsigned long long
pack2(uint32_t lo, uint32_t hi)
{
    return static_cast<unsigned long long>(hi) << 32 | lo;
}

// Claim of a slot whose image is exp (4 words; a never-used slot is all ones) with one compare-and-swap
// over the whole slot: key and mapped value are written together (4, 8 or 16 bytes), so no reader sees
// the key without its value.  Returns true when the claim took the slot; old_key is the key word found.
template <int KIND>
SG_D bool
claim_slot_image(char* p, const uint32_t (&exp)[4], typename kind_consts<KIND>::K key,
                 typename kind_consts<KIND>::V val, typename kind_consts<KIND>::K& old_key)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    constexpr int sb = C::slot_bytes;
    uint32_t nw[4] = { exp[0], exp[1], exp[2], exp[3] };
    nw[0] = static_cast<uint32_t>(key);
    if constexpr (sizeof(K) == 8)
    {
        nw[1] = static_cast<uint32_t>(static_cast<uint64_t>(key) >> 32);
    }
    if constexpr (kind_traits<KIND>::is_map)
    {
        constexpr int vo = kind_traits<KIND>::val_offset / 4;
        nw[vo] = static_cast<uint32_t>(val);
        if constexpr (sizeof(V) == 8)
        {
            nw[vo + 1] = static_cast<uint32_t>(static_cast<uint64_t>(val) >> 32);
        }
    }
    if constexpr (sb == 4)
    {
        const uint32_t o = atomicCAS(reinterpret_cast<unsigned int*>(p), exp[0], nw[0]);
        old_key = static_cast<K>(o);
        return o == exp[0];
    }
    else if constexpr (sb == 8)
    {
        const unsigned long long e = pack2(exp[0], exp[1]);
        const unsigned long long o = atomicCAS(reinterpret_cast<unsigned long long*>(p), e, pack2(nw[0], nw[1]));
        old_key = sizeof(K) == 8 ? static_cast<K>(o) : static_cast<K>(static_cast<uint32_t>(o));
        return o == e;
    }
    else
    {
        const unsigned long long e_lo = pack2(exp[0], exp[1]);
        const unsigned long long e_hi = pack2(exp[2], exp[3]);
        unsigned long long o_lo, o_hi;
        cas128(p, e_lo, e_hi, pack2(nw[0], nw[1]), pack2(nw[2], nw[3]), o_lo, o_hi);
        old_key = sizeof(K) == 8 ? static_cast<K>(o_lo) : static_cast<K>(static_cast<uint32_t>(o_lo));
        return o_lo == e_lo && o_hi == e_hi;
    }
}
#endif

} // namespace detail
} // namespace sg

#endif

// Device-side building blocks of the table kernels (probe groups, tile probing, counters), shared by the
// single-table entry points (unordered.cu) and the batched many-table entry points (batch.cu).
#ifndef SG_TABLE_CORE_CUH
#define SG_TABLE_CORE_CUH

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "stdgpu_gb300/detail/layout.cuh"

namespace sg
{
namespace detail
{

constexpr int kThreads = 256;

// Resident blocks per SM the bulk kernels are compiled for (register budget 65536 / (256 * N)).
#ifndef SG_BULK_MIN_BLOCKS
#define SG_BULK_MIN_BLOCKS 4
#endif
#ifndef SG_FIND_MIN_BLOCKS
#define SG_FIND_MIN_BLOCKS SG_BULK_MIN_BLOCKS
#endif
#ifndef SG_ORDERED_MIN_BLOCKS
#define SG_ORDERED_MIN_BLOCKS SG_BULK_MIN_BLOCKS
#endif
constexpr int kRangeChunk = 2048; // slots per block in the compaction kernels (256 threads x 8 slots)

// Kernel view of a table.  Group and slot indices fit 32 bits (max_size() < 2^31), so the hot paths
// index in 32-bit arithmetic and widen only to form addresses.
struct dview
{
    char* slots;
    table_header* hdr;
    uint32_t num_groups;
    uint32_t total;
    int bits;
};

// ---------------------------------------------------------------- geometry

// bit_ceil over size_t: src/stdgpu/impl/bit_detail.h:36-62
inline uint64_t
bit_ceil_u64(uint64_t x)
{
    uint64_t r = 1;
    while (r < x && r != 0)
    {
        r <<= 1;
    }
    return r;
}

// createDeviceObject geometry: src/stdgpu/impl/unordered_base_detail.cuh:1264-1273 and
// expected_collisions :34-48, evaluated with the same float / long double steps.
inline void
reference_geometry(int64_t capacity, int64_t* bucket_count, int64_t* excess_count)
{
    const float c = std::ceil(static_cast<float>(capacity) / 1.0F);
    const uint64_t b = bit_ceil_u64(static_cast<uint64_t>(c));
    const long double k = static_cast<long double>(b);
    const long double n = static_cast<long double>(capacity);
    const int64_t e = static_cast<int64_t>(std::ceil(n * (1.0L - std::pow(1.0L - (1.0L / k), n - 1.0L))));
    *bucket_count = static_cast<int64_t>(b);
    *excess_count = e + 1;
}

inline int
log2_exact(int64_t x)
{
    int b = 0;
    while ((int64_t{ 1 } << b) < x)
    {
        ++b;
    }
    return b;
}

// ---------------------------------------------------------------- device helpers

// Home group: the reference's bucket(key) scaled from 2^bits buckets onto num_groups groups.
template <int KIND>
SG_D uint32_t
home_of(const dview& t, uint64_t hash)
{
    const uint32_t b = static_cast<uint32_t>(fibonacci_bucket(hash, t.bits));
    return static_cast<uint32_t>((static_cast<uint64_t>(b) * t.num_groups) >> t.bits);
}

SG_D uint32_t
next_group32(uint32_t g, uint32_t num_groups)
{
    return g + 1 == num_groups ? 0u : g + 1;
}

template <int KIND>
SG_D typename kind_consts<KIND>::K
cas_key(const dview& t, uint32_t slot, typename kind_consts<KIND>::K expected, typename kind_consts<KIND>::K desired)
{
    using K = typename kind_consts<KIND>::K;
    char* p = t.slots + static_cast<uint64_t>(slot) * kind_consts<KIND>::slot_bytes;
    if constexpr (sizeof(K) == 8)
    {
        return static_cast<K>(atomicCAS(reinterpret_cast<unsigned long long*>(p),
                                        static_cast<unsigned long long>(expected),
                                        static_cast<unsigned long long>(desired)));
    }
    else
    {
        return static_cast<K>(atomicCAS(reinterpret_cast<unsigned int*>(p),
                                        static_cast<unsigned int>(expected),
                                        static_cast<unsigned int>(desired)));
    }
}

template <int KIND>
SG_D void
store_value(const dview& t, uint32_t slot, typename kind_consts<KIND>::V v)
{
    if constexpr (kind_traits<KIND>::is_map)
    {
        using V = typename kind_consts<KIND>::V;
        *reinterpret_cast<V*>(t.slots + static_cast<uint64_t>(slot) * kind_consts<KIND>::slot_bytes +
                              kind_traits<KIND>::val_offset) = v;
    }
}

// Claim of a free slot with one compare-and-swap over the whole slot -- key and mapped value written
// together (4, 8 or 16 bytes), so no separate store of the value follows and no reader can see the key
// without its value.  A never-used slot is all ones; an erased slot keeps its old value bytes, so for
// it the expected image is read first (erased marker in the key word, the bytes found elsewhere).
// Returns true when the claim took the slot; old_key is the key word found there.
template <int KIND>
SG_D bool
claim_slot(const dview& t, uint32_t slot, bool erased, typename kind_consts<KIND>::K key,
           typename kind_consts<KIND>::V val, typename kind_consts<KIND>::K& old_key)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    constexpr int sb = C::slot_bytes;
    char* p = t.slots + static_cast<uint64_t>(slot) * sb;
    uint32_t exp[4] = { ~0u, ~0u, ~0u, ~0u };
    if (erased)
    {
        if constexpr (sb == 16)
        {
            const uint4 w = __ldcg(reinterpret_cast<const uint4*>(p));
            exp[1] = w.y;
            exp[2] = w.z;
            exp[3] = w.w;
        }
        else if constexpr (sb == 8)
        {
            exp[1] = __ldcg(reinterpret_cast<const unsigned int*>(p) + 1);
        }
        exp[0] = static_cast<uint32_t>(C::tomb_key);
        if constexpr (sizeof(K) == 8)
        {
            exp[1] = static_cast<uint32_t>(static_cast<uint64_t>(C::tomb_key) >> 32);
        }
    }
    return claim_slot_image<KIND>(p, exp, key, val, old_key);
}

// Input element i: value_type array (AoS) or separate key / mapped arrays.
template <int KIND, bool AOS>
SG_D void
load_input(const void* in0, const void* in1, int64_t i, typename kind_consts<KIND>::K& key,
           typename kind_consts<KIND>::V& val)
{
    using K = typename kind_consts<KIND>::K;
    using V = typename kind_consts<KIND>::V;
    constexpr int sb = kind_consts<KIND>::slot_bytes;
    if constexpr (AOS)
    {
        if constexpr (sb == 16)
        {
            const uint4 d = __ldcs(reinterpret_cast<const uint4*>(in0) + i);
            key = key_in_lane<KIND>(d, 0);
            val = value_in_lane<KIND>(d, 0);
        }
        else if constexpr (sb == 8)
        {
            const uint2 d = __ldcs(reinterpret_cast<const uint2*>(in0) + i);
            const uint4 q = make_uint4(d.x, d.y, 0u, 0u);
            key = key_in_lane<KIND>(q, 0);
            val = value_in_lane<KIND>(q, 0);
        }
        else
        {
            key = static_cast<K>(__ldcs(reinterpret_cast<const unsigned int*>(in0) + i));
            val = V{};
        }
    }
    else
    {
        key = __ldcs(reinterpret_cast<const K*>(in0) + i);
        if constexpr (kind_traits<KIND>::is_map)
        {
            val = in1 != nullptr ? __ldcs(reinterpret_cast<const V*>(in1) + i) : V{};
        }
        else
        {
            val = V{};
        }
    }
}

// Out-of-band keys (EMPTY- or TOMB-valued): presence in the header, storage in the tail group.
template <int KIND>
SG_D int
special_insert(const dview& t, typename kind_consts<KIND>::K key, typename kind_consts<KIND>::V val)
{
    using C = kind_consts<KIND>;
    const int s = key == C::empty_key ? 0 : 1;
    if (atomicCAS(&t.hdr->special_state[s], 0u, 2u) != 0u)
    {
        return 0;
    }
    const uint32_t slot = t.num_groups * C::slots_per_group + s;
    *reinterpret_cast<typename C::K*>(t.slots + static_cast<uint64_t>(slot) * C::slot_bytes) = key;
    store_value<KIND>(t, slot, val);
    __threadfence();
    atomicExch(&t.hdr->special_state[s], 1u);
    return 1;
}

template <int KIND>
SG_D bool
special_find(const dview& t, typename kind_consts<KIND>::K key, typename kind_consts<KIND>::V& val)
{
    using C = kind_consts<KIND>;
    const int s = key == C::empty_key ? 0 : 1;
    if (*reinterpret_cast<volatile unsigned*>(&t.hdr->special_state[s]) != 1u)
    {
        return false;
    }
    const uint64_t slot = static_cast<uint64_t>(t.num_groups) * C::slots_per_group + s;
    if constexpr (kind_traits<KIND>::is_map)
    {
        val = *reinterpret_cast<const volatile typename C::V*>(t.slots + slot * C::slot_bytes +
                                                               kind_traits<KIND>::val_offset);
    }
    return true;
}

template <int KIND>
SG_D int
special_erase(const dview& t, typename kind_consts<KIND>::K key)
{
    using C = kind_consts<KIND>;
    const int s = key == C::empty_key ? 0 : 1;
    return atomicCAS(&t.hdr->special_state[s], 1u, 0u) == 1u ? 1 : 0;
}

// ---------------------------------------------------------------- tile probing
// A tile of 4 lanes owns one key at a time.  Lane q of the tile reads sector q (bytes 32q..32q+31) of
// the key's 128-byte probe group with one 256-bit load, so each group costs one 128-byte request and a
// warp instruction covers 8 keys.  Measured on GB300 over an 8 GB buffer, random 128-byte lines read
// this way reach 36-38 G lines/s, against 21-25 G with 8 lanes x 16 B and 10-12 G with one thread
// issuing 4 x 32 B.

constexpr int kTile = 4;

SG_D void
load_sector(const dview& t, uint32_t g, int q, uint32_t (&w)[8])
{
    const char* p = t.slots + (static_cast<uint64_t>(g) << 7) + 32 * q;
    asm volatile("ld.global.cg.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(w[0]), "=r"(w[1]), "=r"(w[2]), "=r"(w[3]), "=r"(w[4]), "=r"(w[5]), "=r"(w[6]), "=r"(w[7])
                 : "l"(p));
}

template <int KIND>
struct sector_consts
{
    static constexpr int slot_words = kind_consts<KIND>::slot_bytes / 4;
    static constexpr int slots = 32 / kind_consts<KIND>::slot_bytes; // slots per 32-byte sector
};

template <int KIND>
SG_D typename kind_consts<KIND>::K
sector_key(const uint32_t (&w)[8], int s)
{
    using K = typename kind_consts<KIND>::K;
    constexpr int sw = sector_consts<KIND>::slot_words;
    if constexpr (sizeof(K) == 8)
    {
        return static_cast<uint64_t>(w[sw * s + 1]) << 32 | w[sw * s];
    }
    else
    {
        return static_cast<K>(w[sw * s]);
    }
}

template <int KIND>
SG_D typename kind_consts<KIND>::V
sector_value(const uint32_t (&w)[8], int s)
{
    using V = typename kind_consts<KIND>::V;
    constexpr int sw = sector_consts<KIND>::slot_words;
    constexpr int off = kind_traits<KIND>::val_offset / 4;
    if constexpr (!kind_traits<KIND>::is_map)
    {
        return V{};
    }
    else if constexpr (sizeof(V) == 8)
    {
        return static_cast<uint64_t>(w[sw * s + off + 1]) << 32 | w[sw * s + off];
    }
    else
    {
        return static_cast<V>(w[sw * s + off]);
    }
}

// Bit s set when sector slot s holds key / is never-used / is erased and below total (reusable).
template <int KIND, bool WANT_TOMB>
SG_D void
sector_masks(const uint32_t (&w)[8], typename kind_consts<KIND>::K key, uint32_t first_slot, uint32_t total,
             unsigned& m_match, unsigned& m_empty, unsigned& m_tomb)
{
    using C = kind_consts<KIND>;
    constexpr int S = sector_consts<KIND>::slots;
    m_match = 0;
    m_empty = 0;
    m_tomb = 0;
#pragma unroll
    for (int s = 0; s < S; ++s)
    {
        const typename C::K k = sector_key<KIND>(w, s);
        m_match |= static_cast<unsigned>(k == key) << s;
        m_empty |= static_cast<unsigned>(k == C::empty_key) << s;
        if constexpr (WANT_TOMB)
        {
            m_tomb |= static_cast<unsigned>(k == C::tomb_key) << s;
        }
    }
    if constexpr (WANT_TOMB)
    {
        // slots at or above total_count are never claimed
        if (first_slot + S > total)
        {
            m_tomb &= first_slot >= total ? 0u : ((1u << (total - first_slot)) - 1u);
        }
    }
}

template <int KIND>
SG_D typename kind_consts<KIND>::V
select_sector_value(const uint32_t (&w)[8], unsigned one_hot)
{
    typename kind_consts<KIND>::V v{};
#pragma unroll
    for (int s = 0; s < sector_consts<KIND>::slots; ++s)
    {
        if (one_hot & (1u << s))
        {
            v = sector_value<KIND>(w, s);
        }
    }
    return v;
}

// Per-key rotation of the slot order inside a group.  Every insert of a key takes, within a group, the
// first free slot at or after slot rot_of(hash) (cyclically), where the reference-compatible rule would take
// the first free slot.  Copies of one key follow the same order, so the duplicate argument below holds
// unchanged, and concurrent inserts of different keys into one group start at different slots instead of
// all racing for its first free slot.  Lookups scan whole groups, so they do not depend on the order.
SG_D uint32_t
rot_of(uint64_t hash)
{
    return static_cast<uint32_t>((hash * 0xD6E8FEB86659FD93ull) >> 59);
}

// Index of the first set bit of the G-bit mask m at or after bit o, cyclically; -1 when m is empty.
template <uint32_t G>
SG_D int
first_from(unsigned m, uint32_t o)
{
    if (m == 0u)
    {
        return -1;
    }
    o &= G - 1;
    unsigned r;
    if constexpr (G == 32)
    {
        r = __funnelshift_r(m, m, o);
    }
    else
    {
        r = ((m >> o) | (m << (G - o))) & ((1u << G) - 1u);
    }
    return static_cast<int>((static_cast<uint32_t>(__ffs(r) - 1) + o) & (G - 1));
}

// G-bit mask of a group from the tile's four S-bit sector masks (lane q holds sector q).
template <uint32_t S>
SG_D unsigned
group_mask(unsigned sector_mask, int q, unsigned mask)
{
    unsigned g = sector_mask << (q * S);
    g |= __shfl_xor_sync(mask, g, 1);
    g |= __shfl_xor_sync(mask, g, 2);
    return g;
}

// Insert of one key by one tile (all 4 lanes call it with the same key; w is this lane's sector of the
// key's home group).  Returns 1 inserted, 0 already present, 2 refused (no free slot in the table),
// 3 retry limit.  With REUSE, erased slots are claimed too: the tile scans to the first group holding a
// never-used slot (so a copy of the key stored beyond an erased slot is seen) and claims the first free
// slot of the probe sequence.  Free slots only disappear during an insert launch, so two inserts of one
// key cannot both succeed: each has read every slot before the one it claims.
template <int KIND, bool REUSE>
SG_D int
tile_insert(const dview& t, typename kind_consts<KIND>::K key, typename kind_consts<KIND>::V val, uint32_t home,
            uint32_t (&w)[8], unsigned tmask, int tbase, int q, unsigned int& tombs_reused, uint32_t rot)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    constexpr uint32_t G = C::slots_per_group;
    constexpr uint32_t S = sector_consts<KIND>::slots;
    uint32_t g = home;
    int32_t free_slot = -1;
    uint32_t probes = 0;
    int retries = 0;
    while (true)
    {
        unsigned mm, me, mt;
        sector_masks<KIND, REUSE>(w, key, g * G + q * S, t.total, mm, me, mt);
        if (__ballot_sync(tmask, mm != 0u) != 0u)
        {
            return 0;
        }
        if constexpr (REUSE)
        {
            if (free_slot < 0)
            {
                const int s = first_from<G>(group_mask<S>(mt, q, tmask), rot);
                if (s >= 0)
                {
                    free_slot = static_cast<int32_t>(g * G + static_cast<uint32_t>(s));
                }
            }
        }
        const unsigned ge = group_mask<S>(me, q, tmask);
        bool claim = ge != 0u;
        if (!claim && ++probes >= t.num_groups)
        {
            if (!(REUSE && free_slot >= 0))
            {
                return 2;
            }
            claim = true; // no never-used slot anywhere: take the first erased slot seen
        }
        if (!claim)
        {
            g = next_group32(g, t.num_groups);
            load_sector(t, g, q, w);
            continue;
        }
        uint32_t target;
        K expected;
        if (REUSE && free_slot >= 0)
        {
            target = static_cast<uint32_t>(free_slot);
            expected = C::tomb_key;
        }
        else
        {
            target = g * G + static_cast<uint32_t>(first_from<G>(ge, rot));
            expected = C::empty_key;
        }
        K old = expected;
        if (q == 0)
        {
            old = cas_key<KIND>(t, target, expected, key);
            if (old == expected)
            {
                store_value<KIND>(t, target, val);
                tombs_reused += (expected == C::tomb_key);
            }
        }
        old = __shfl_sync(tmask, old, tbase);
        if (old == expected)
        {
            return 1;
        }
        if (old == key)
        {
            return 0;
        }
        // another key took the slot: rescan from the slot's group (every earlier group was seen without
        // a free slot)
        if (++retries > 65536)
        {
            return 3;
        }
        g = target / G;
        probes = g >= home ? g - home : g + t.num_groups - home;
        free_slot = -1;
        load_sector(t, g, q, w);
    }
}

// Slot of key (mapped value broadcast to the tile through val), or -1.  Stops at the first group
// holding a never-used slot.
template <int KIND>
SG_D int32_t
tile_find(const dview& t, typename kind_consts<KIND>::K key, uint32_t home, uint32_t (&w)[8], unsigned tmask,
          int tbase, int q, typename kind_consts<KIND>::V& val)
{
    constexpr uint32_t G = kind_consts<KIND>::slots_per_group;
    constexpr uint32_t S = sector_consts<KIND>::slots;
    uint32_t g = home;
    for (uint32_t probes = 0; probes < t.num_groups; ++probes)
    {
        unsigned mm, me, mt;
        sector_masks<KIND, false>(w, key, 0, 0, mm, me, mt);
        const unsigned bm = __ballot_sync(tmask, mm != 0u);
        if (bm != 0u)
        {
            const int owner = __ffs(bm) - 1;
            typename kind_consts<KIND>::V mine{};
            if constexpr (kind_traits<KIND>::is_map)
            {
                mine = select_sector_value<KIND>(w, mm);
            }
            val = __shfl_sync(tmask, mine, owner);
            const int s = __ffs(__shfl_sync(tmask, mm, owner)) - 1;
            return static_cast<int32_t>(g * G + (owner - tbase) * S + s);
        }
        if (__ballot_sync(tmask, me != 0u) != 0u)
        {
            return -1;
        }
        g = next_group32(g, t.num_groups);
        load_sector(t, g, q, w);
    }
    return -1;
}

// ---------------------------------------------------------------- block reduction of counters

template <int N>
SG_D void
block_add(unsigned long long (&v)[N], unsigned long long* const (&dst)[N])
{
    __shared__ unsigned long long red[N][kThreads / 32];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < N; ++k)
    {
        unsigned long long x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1)
        {
            x += __shfl_xor_sync(0xffffffffu, x, o);
        }
        if (lane == 0)
        {
            red[k][warp] = x;
        }
    }
    __syncthreads();
    if (threadIdx.x < N)
    {
        unsigned long long s = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w)
        {
            s += red[threadIdx.x][w];
        }
        if (s != 0 && dst[threadIdx.x] != nullptr)
        {
            atomicAdd(dst[threadIdx.x], s);
        }
    }
}

// Lanes of a warp: tiles of 4; the warp holds 32 keys (one per lane, loaded coalesced) and each tile
// resolves the 4 keys of its own lanes in 4 rounds, after issuing the home-group loads of all 4.
struct tile_lanes
{
    int lane, tbase, q;
    unsigned tmask;
    SG_D tile_lanes()
    {
        lane = threadIdx.x & 31;
        tbase = lane & ~(kTile - 1);
        q = lane & (kTile - 1);
        tmask = 0xFu << tbase;
    }
};


// Counts of one lane over the steps it ran.
// 32-bit: a lane's count between two flushes stays far below 2^32, and registers are what bounds how
// many warps the probe kernels keep in flight.
struct step_counts
{
    unsigned int done = 0;    // inserted / erased
    unsigned int refused = 0; // inserts refused: no free slot left
    unsigned int reused = 0;  // erased slots claimed by inserts
    unsigned int oob = 0;     // erased out-of-band keys
    unsigned int retry = 0;   // retry limit reached
};

// ---------------------------------------------------------------- warp steps
// One step covers 32 consecutive elements (lane l owns element i; valid when i is in range), all on
// table t, and is called by all 32 lanes of the warp together.  Each tile of 4 lanes loads the home
// groups of its 4 keys (4 x 128-byte requests per tile, 32 per warp).  Each group is then resolved
// with full-warp ballots: nibble `tbase` of a ballot is the tile's view of its group (bit q = sector
// q), so the common case -- the key's fate is decided in its home group -- runs without any branch
// that differs between tiles.  Only keys whose home group is full of other keys (or whose claim lost
// to another key) take the tile-cooperative slow path.

SG_D unsigned
tile_nibble(unsigned ballot, int tbase)
{
    return (ballot >> tbase) & 0xFu;
}

// Loads the home groups of the tile's 4 keys; a lane with nothing to probe reports home 0 (a valid
// group, read and ignored).
template <int KIND>
SG_D void
load_homes(const dview& t, const tile_lanes& L, uint64_t hash, bool probe, uint32_t (&hr)[kTile],
           uint32_t (&pre)[kTile][8])
{
    const uint32_t home = probe ? home_of<KIND>(t, hash) : 0u;
#pragma unroll
    for (int r = 0; r < kTile; ++r)
    {
        hr[r] = __shfl_sync(0xffffffffu, home, L.tbase + r);
        load_sector(t, hr[r], L.q, pre[r]);
    }
}

// Insert step.  Per key, from its home group: present (nothing to do), or a claim of the first erased
// slot of the group (when the group also has a never-used slot) else of the first never-used slot, made
// by the key's own lane with one compare-and-swap -- 32 claims in flight per warp.
// The step over keys already in registers (key / val of lane element i, meaningful when valid; hashes as
// in the loading steps below).
// GIVEN: the caller passes the key's hash in given_hash (a staged element that carries it).
template <int KIND, bool GIVEN = false>
SG_D void
insert_kv_step(const dview& t, const tile_lanes& L, typename kind_consts<KIND>::K key,
               typename kind_consts<KIND>::V val, int64_t i, bool valid, uint8_t* out_flags, step_counts& c,
               const uint64_t* hashes = nullptr, uint64_t given_hash = 0)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    constexpr uint32_t G = C::slots_per_group;
    constexpr uint32_t S = sector_consts<KIND>::slots;
    if (!valid)
    {
        key = C::empty_key;
        val = V{};
    }
    const bool special = valid && key >= C::tomb_key;
    int res = special ? special_insert<KIND>(t, key, val) : 0;
    const bool probe = valid && !special;
    uint32_t hr[kTile];
    uint32_t pre[kTile][8];
    const uint64_t hash = GIVEN ? given_hash
                                : (hashes != nullptr && probe ? __ldcs(hashes + i) : static_cast<uint64_t>(key));
    load_homes<KIND>(t, L, hash, probe, hr, pre);
    int my_state = 0; // 0 present, 1 claim my_target, 2 decided beyond the home group
    uint32_t my_target = 0;
    bool my_tomb = false;
    unsigned my_free = 0u; // never-used slots of the home group as read (bit = slot within the group)
    const uint32_t my_rot = rot_of(hash);
#pragma unroll
    for (int r = 0; r < kTile; ++r)
    {
        const K kr = __shfl_sync(0xffffffffu, key, L.tbase + r);
        const uint32_t rot = __shfl_sync(0xffffffffu, my_rot, L.tbase + r);
        unsigned mm, me, mt;
        sector_masks<KIND, true>(pre[r], kr, hr[r] * G + L.q * S, t.total, mm, me, mt);
        const unsigned tm = tile_nibble(__ballot_sync(0xffffffffu, mm != 0u), L.tbase);
        // the group's never-used and erased slots, gathered from the tile's 4 sectors
        const unsigned gfree = group_mask<S>(me, L.q, 0xffffffffu);
        const unsigned gtomb = group_mask<S>(mt, L.q, 0xffffffffu);
        const bool tomb = gtomb != 0u;
        const int s_claim = first_from<G>(tomb ? gtomb : gfree, rot);
        const uint32_t target = hr[r] * G + static_cast<uint32_t>(s_claim < 0 ? 0 : s_claim);
        const int state = tm != 0u ? 0 : (gfree != 0u ? 1 : 2);
        if (L.q == r)
        {
            my_state = state;
            my_target = target;
            my_tomb = tomb;
            my_free = gfree;
        }
    }
    bool again = false;
    if (probe && my_state == 1)
    {
        K old;
        if (claim_slot<KIND>(t, my_target, my_tomb, key, val, old))
        {
            c.reused += my_tomb ? 1u : 0u;
            res = 1;
        }
        else if (old != key)
        {
            // Lost the slot to another key.  Without erased slots in the group, try its next never-used
            // slots as read: every slot before each of them holds another key (read so, or returned by a
            // failed claim), so a claim there keeps the first-free-slot rule; a returned copy of this key
            // means present.  Whatever is left goes to the tile's slow path.
            again = true;
            if (!my_tomb)
            {
                const uint32_t gbase = my_target - my_target % G;
                unsigned rest = my_free & ~(1u << (my_target - gbase));
                while (rest != 0u)
                {
                    const uint32_t s = static_cast<uint32_t>(first_from<G>(rest, my_rot));
                    const uint32_t slot = gbase + s;
                    rest &= ~(1u << s);
                    if (claim_slot<KIND>(t, slot, false, key, val, old))
                    {
                        res = 1;
                        again = false;
                        break;
                    }
                    if (old == key)
                    {
                        again = false;
                        break;
                    }
                }
            }
        }
    }
    again = again || (probe && my_state == 2);
    const unsigned aball = __ballot_sync(0xffffffffu, again);
    if (aball != 0u)
    {
        const unsigned amask = tile_nibble(aball, L.tbase);
#pragma unroll 1
        for (int r = 0; r < kTile; ++r)
        {
            if (amask & (1u << r))
            {
                const K kr = __shfl_sync(L.tmask, key, L.tbase + r);
                const V vr = __shfl_sync(L.tmask, val, L.tbase + r);
                uint32_t w[8];
                load_sector(t, hr[r], L.q, w);
                const uint32_t rot = __shfl_sync(L.tmask, my_rot, L.tbase + r);
                const int x = tile_insert<KIND, true>(t, kr, vr, hr[r], w, L.tmask, L.tbase, L.q, c.reused, rot);
                if (L.q == r)
                {
                    res = x;
                }
            }
        }
    }
    if (valid)
    {
        c.done += (res == 1);
        c.refused += (res == 2);
        c.retry += (res == 3);
        if (out_flags != nullptr)
        {
            out_flags[i] = static_cast<uint8_t>(res == 1);
        }
    }
}

template <int KIND, bool AOS>
SG_D void
insert_step(const dview& t, const tile_lanes& L, const void* in0, const void* in1, int64_t i, bool valid,
            uint8_t* out_flags, step_counts& c, const uint64_t* hashes = nullptr)
{
    typename kind_consts<KIND>::K key = kind_consts<KIND>::empty_key;
    typename kind_consts<KIND>::V val{};
    if (valid)
    {
        load_input<KIND, AOS>(in0, in1, i, key, val);
    }
    insert_kv_step<KIND>(t, L, key, val, i, valid, out_flags, c, hashes);
}

// Locates the slot of each lane's key (-1 when absent); with WANT_VALUE the mapped value comes back in
// val.  Keys not decided in their home group (group full of other keys) continue with tile_find.
template <int KIND, bool WANT_VALUE>
SG_D int32_t
locate_step(const dview& t, const tile_lanes& L, typename kind_consts<KIND>::K key, uint64_t hash, bool probe,
            typename kind_consts<KIND>::V& val)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    constexpr uint32_t G = C::slots_per_group;
    constexpr uint32_t S = sector_consts<KIND>::slots;
    uint32_t hr[kTile];
    uint32_t pre[kTile][8];
    load_homes<KIND>(t, L, hash, probe, hr, pre);
    int32_t my_slot = -1;
    bool my_more = false;
#pragma unroll
    for (int r = 0; r < kTile; ++r)
    {
        const K kr = __shfl_sync(0xffffffffu, key, L.tbase + r);
        unsigned mm, me, mt;
        sector_masks<KIND, false>(pre[r], kr, 0, 0, mm, me, mt);
        const unsigned tm = tile_nibble(__ballot_sync(0xffffffffu, mm != 0u), L.tbase);
        const unsigned te = tile_nibble(__ballot_sync(0xffffffffu, me != 0u), L.tbase);
        const int owner = (__ffs(tm) - 1) & (kTile - 1);
        const unsigned om = __shfl_sync(0xffffffffu, mm, L.tbase + owner);
        V vr{};
        if constexpr (WANT_VALUE && kind_traits<KIND>::is_map)
        {
            vr = __shfl_sync(0xffffffffu, select_sector_value<KIND>(pre[r], mm), L.tbase + owner);
        }
        const int32_t slot = tm != 0u ? static_cast<int32_t>(hr[r] * G + static_cast<uint32_t>(owner) * S +
                                                             static_cast<uint32_t>(__ffs(om) - 1))
                                      : -1;
        if (L.q == r)
        {
            my_slot = slot;
            my_more = tm == 0u && te == 0u;
            val = vr;
        }
    }
    const unsigned mball = __ballot_sync(0xffffffffu, probe && my_more);
    if (mball != 0u)
    {
        const unsigned mmask = tile_nibble(mball, L.tbase);
#pragma unroll 1
        for (int r = 0; r < kTile; ++r)
        {
            if (mmask & (1u << r))
            {
                const K kr = __shfl_sync(L.tmask, key, L.tbase + r);
                const uint32_t g = next_group32(hr[r], t.num_groups);
                uint32_t w[8];
                load_sector(t, g, L.q, w);
                V vr{};
                const int32_t slot = tile_find<KIND>(t, kr, g, w, L.tmask, L.tbase, L.q, vr);
                if (L.q == r)
                {
                    my_slot = slot;
                    val = vr;
                }
            }
        }
    }
    return probe ? my_slot : -1;
}

// Erase step: every lane locates its key, then swaps its slot to the erased marker.
template <int KIND, bool GIVEN = false>
SG_D void
erase_key_step(const dview& t, const tile_lanes& L, typename kind_consts<KIND>::K key, int64_t i, bool valid,
               uint8_t* out_flags, step_counts& c, const uint64_t* hashes = nullptr, uint64_t given_hash = 0)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    if (!valid)
    {
        key = C::empty_key;
    }
    const bool special = valid && key >= C::tomb_key;
    int res = 0;
    if (special)
    {
        res = special_erase<KIND>(t, key);
        c.oob += static_cast<unsigned int>(res);
    }
    const bool probe = valid && !special;
    V dummy{};
    const uint64_t hash = GIVEN ? given_hash
                                : (hashes != nullptr && probe ? __ldcs(hashes + i) : static_cast<uint64_t>(key));
    const int32_t my_slot = locate_step<KIND, false>(t, L, key, hash, probe, dummy);
    if (my_slot >= 0)
    {
        res = cas_key<KIND>(t, static_cast<uint32_t>(my_slot), key, C::tomb_key) == key ? 1 : 0;
    }
    if (valid)
    {
        c.done += static_cast<unsigned int>(res);
        if (out_flags != nullptr)
        {
            out_flags[i] = static_cast<uint8_t>(res);
        }
    }
}

// Erase step whose compare-and-swap result is consumed one step later: the swap of step k stays in flight
// while step k + 1 issues its home-group loads, so a warp waits once per step instead of twice.  For calls
// without per-key flags; the caller adds the last step's result with erase_pending_done.
template <int KIND>
struct erase_pending
{
    typename kind_consts<KIND>::K key{};
    typename kind_consts<KIND>::K old{};
    bool live = false;
};

template <int KIND>
SG_D unsigned int
erase_pending_done(const erase_pending<KIND>& p)
{
    return p.live && p.old == p.key ? 1u : 0u;
}

template <int KIND>
SG_D void
erase_key_step_deferred(const dview& t, const tile_lanes& L, typename kind_consts<KIND>::K key, bool valid,
                        step_counts& c, erase_pending<KIND>& pend)
{
    using C = kind_consts<KIND>;
    using V = typename C::V;
    if (!valid)
    {
        key = C::empty_key;
    }
    const bool special = valid && key >= C::tomb_key;
    if (special)
    {
        const unsigned int r = static_cast<unsigned int>(special_erase<KIND>(t, key));
        c.oob += r;
        c.done += r;
    }
    const bool probe = valid && !special;
    V dummy{};
    const int32_t my_slot = locate_step<KIND, false>(t, L, key, static_cast<uint64_t>(key), probe, dummy);
    c.done += erase_pending_done<KIND>(pend);
    pend.live = my_slot >= 0;
    pend.key = key;
    if (pend.live)
    {
        pend.old = cas_key<KIND>(t, static_cast<uint32_t>(my_slot), key, C::tomb_key);
    }
}

template <int KIND>
SG_D void
erase_step(const dview& t, const tile_lanes& L, const void* keys, int64_t i, bool valid, uint8_t* out_flags,
           step_counts& c, const uint64_t* hashes = nullptr)
{
    using K = typename kind_consts<KIND>::K;
    const K key = valid ? __ldcs(reinterpret_cast<const K*>(keys) + i) : kind_consts<KIND>::empty_key;
    erase_key_step<KIND>(t, L, key, i, valid, out_flags, c, hashes);
}

// Find / contains step.
template <int KIND, bool WANT_VALUES>
SG_D void
find_key_step(const dview& t, const tile_lanes& L, typename kind_consts<KIND>::K key, int64_t i, bool valid,
              void* out_vals, uint8_t* out_found, const uint64_t* hashes = nullptr)
{
    using C = kind_consts<KIND>;
    using K = typename C::K;
    using V = typename C::V;
    if (!valid)
    {
        key = C::empty_key;
    }
    const bool special = valid && key >= C::tomb_key;
    V val{};
    bool found = special ? special_find<KIND>(t, key, val) : false;
    const bool probe = valid && !special;
    V pv{};
    const uint64_t hash = hashes != nullptr && probe ? __ldcs(hashes + i) : static_cast<uint64_t>(key);
    const int32_t slot = locate_step<KIND, WANT_VALUES>(t, L, key, hash, probe, pv);
    if (probe)
    {
        found = slot >= 0;
        val = pv;
    }
    if (valid)
    {
        if (out_found != nullptr)
        {
            __stcs(out_found + i, static_cast<uint8_t>(found));
        }
        if constexpr (WANT_VALUES && kind_traits<KIND>::is_map)
        {
            if (found && out_vals != nullptr)
            {
                __stcs(reinterpret_cast<V*>(out_vals) + i, val);
            }
        }
    }
}

template <int KIND, bool WANT_VALUES>
SG_D void
find_step(const dview& t, const tile_lanes& L, const void* keys, int64_t i, bool valid, void* out_vals,
          uint8_t* out_found, const uint64_t* hashes = nullptr)
{
    using K = typename kind_consts<KIND>::K;
    const K key = valid ? __ldcs(reinterpret_cast<const K*>(keys) + i) : kind_consts<KIND>::empty_key;
    find_key_step<KIND, WANT_VALUES>(t, L, key, i, valid, out_vals, out_found, hashes);
}

} // namespace detail
} // namespace sg

#endif

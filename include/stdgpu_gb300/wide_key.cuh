// unordered_map<Key, T, Hash> / unordered_set<Key, Hash> for the element types the library's precompiled
// kinds cannot hold: keys of 9 to 16 bytes (a 3 x int32 coordinate, the key of the reference's
// nontrivial-type tests, tests/stdgpu/unordered_map.inc:132-161 and :238-239), and mapped types that are
// not 4- or 8-byte words or not trivially copyable (an empty tag, a float4, a type with a destructor).
//
// Storage, all in this header and instantiated in the caller's translation unit with the caller's types:
//   keys    key words (4, 8 or 16 bytes: the key's object bytes, zero-padded) in 128-byte probe groups,
//           num_groups x G slots, then two out-of-band slots for keys whose word equals one of the two
//           reserved patterns (only keys that fill their word can);
//   values  the mapped objects, one per slot index (maps with a non-empty mapped type), constructed in
//           place when a key takes its slot and destroyed when it leaves it, as the reference constructs
//           and destroys value_type (src/stdgpu/impl/unordered_base_detail.cuh:708-809, :811-913, :1220-1252);
//   header  element count, out-of-band states, sticky error bits.
// Geometry (bucket_count, max_size) and the home group of a key (fibonacci hashing of Hash(key),
// src/stdgpu/impl/unordered_base_detail.cuh:56-85, :547-564, scaled onto the groups) are those of the
// library's own tables, and so are the slot rules: a never-used word is all ones, an erased word all ones
// minus one; a key lives in the first group of its probe chain that had a never-used slot when it was
// inserted, so a lookup stops at the first group with a never-used slot; an insert may take an erased slot
// of that group (or, once no never-used slot is left anywhere, the first erased slot of its chain).  Device
// inserts, which may run beside device erases, hold the stripe lock of the key's home group while they scan
// and claim, so two device inserts of one key are ordered (the reference locks the bucket,
// src/stdgpu/impl/unordered_base_detail.cuh:708-809).
//
// Keys compare with KeyEqual, as the reference compares them on every probe
// (src/stdgpu/impl/unordered_base_detail.cuh:661, :673): a probe accepts a stored key when KeyEqual holds for
// it and the probed key, a lost claim whose winner holds an equal key means present, and an erase swaps out
// the stored word it found.  KeyEqual = void compares the key bytes (the default comparison of keys whose
// equal values have equal bytes).  Keys whose bytes fill their word with all ones or all ones minus one
// (the two reserved patterns, held out of band) compare by their bytes.  The mapped value of a key claimed
// in the same launch as a lookup of it may not be written yet when the lookup reads it.
#ifndef STDGPU_GB300_WIDE_KEY_CUH
#define STDGPU_GB300_WIDE_KEY_CUH

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <new>
#include <type_traits>

namespace stdgpu
{
namespace detail
{

// 16-byte key word; lo holds bytes 0-7 of the key.
struct alignas(16) word128
{
    unsigned long long lo;
    unsigned long long hi;
};

__host__ __device__ inline bool
operator==(const word128& a, const word128& b)
{
    return a.lo == b.lo && a.hi == b.hi;
}

__host__ __device__ inline bool
operator!=(const word128& a, const word128& b)
{
    return !(a == b);
}

template <typename Key>
using wide_word_of =
        std::conditional_t<sizeof(Key) <= 4, std::uint32_t, std::conditional_t<sizeof(Key) <= 8, std::uint64_t, word128>>;

// Reserved patterns, coherent loads (L2, never a stale L1 line) and compare-and-swap of one key word.
template <typename W>
struct wide_word;

template <>
struct wide_word<std::uint32_t>
{
    __host__ __device__ static std::uint32_t
    empty()
    {
        return 0xffffffffu;
    }
    __host__ __device__ static std::uint32_t
    tomb()
    {
        return 0xfffffffeu;
    }
#if defined(__CUDACC__)
    __device__ static std::uint32_t
    load(const std::uint32_t* p)
    {
        std::uint32_t v;
        asm volatile("ld.global.cg.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
        return v;
    }
    __device__ static std::uint32_t
    cas(std::uint32_t* p, std::uint32_t expected, std::uint32_t desired)
    {
        return atomicCAS(reinterpret_cast<unsigned int*>(p), expected, desired);
    }
#endif
};

template <>
struct wide_word<std::uint64_t>
{
    __host__ __device__ static std::uint64_t
    empty()
    {
        return ~std::uint64_t{ 0 };
    }
    __host__ __device__ static std::uint64_t
    tomb()
    {
        return ~std::uint64_t{ 0 } - 1;
    }
#if defined(__CUDACC__)
    __device__ static std::uint64_t
    load(const std::uint64_t* p)
    {
        unsigned long long v;
        asm volatile("ld.global.cg.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
        return v;
    }
    __device__ static std::uint64_t
    cas(std::uint64_t* p, std::uint64_t expected, std::uint64_t desired)
    {
        return atomicCAS(reinterpret_cast<unsigned long long*>(p), static_cast<unsigned long long>(expected),
                         static_cast<unsigned long long>(desired));
    }
#endif
};

template <>
struct wide_word<word128>
{
    __host__ __device__ static word128
    empty()
    {
        return word128{ ~0ull, ~0ull };
    }
    __host__ __device__ static word128
    tomb()
    {
        return word128{ ~0ull - 1, ~0ull };
    }
#if defined(__CUDACC__)
    __device__ static word128
    load(const word128* p)
    {
        word128 v;
        asm volatile("ld.global.cg.v2.u64 {%0, %1}, [%2];" : "=l"(v.lo), "=l"(v.hi) : "l"(p) : "memory");
        return v;
    }
    __device__ static word128
    cas(word128* p, const word128& expected, const word128& desired)
    {
        word128 old;
        sg::detail::cas128(p, expected.lo, expected.hi, desired.lo, desired.hi, old.lo, old.hi);
        return old;
    }
#endif
};

template <typename W, typename Key>
__host__ __device__ inline W
to_wide(const Key& key)
{
    W w{};
    std::memcpy(reinterpret_cast<char*>(&w), reinterpret_cast<const char*>(&key), sizeof(Key));
    return w;
}

template <typename Key, typename W>
__host__ __device__ inline Key
from_wide(const W& w)
{
    Key key;
    std::memcpy(reinterpret_cast<char*>(&key), reinterpret_cast<const char*>(&w), sizeof(Key));
    return key;
}

struct wide_header
{
    unsigned long long size;       // stored elements, out-of-band keys included
    unsigned int special_state[2]; // out-of-band key [0] all-ones, [1] all-ones minus one: 0 absent, 1 present, 2 busy
    unsigned int error;            // sticky error bits (sg::detail::kErrRetry)
    unsigned int bad;              // valid(): invariants found broken
    unsigned long long count;      // valid() / device_range() scratch counter
};

constexpr int kWideRetry = 1 << 16; // re-reads of one group after lost claims before a call gives up

template <typename T>
struct wide_mapped_store
{
    static constexpr bool stored = !std::is_void<T>::value && !std::is_empty<T>::value;
};
template <>
struct wide_mapped_store<void>
{
    static constexpr bool stored = false;
};

struct wide_insert_result
{
    std::int64_t slot; // the key's slot, or -1 when refused
    bool inserted;
};

// Word j of a 16-byte load {a, b}.
template <typename W>
__host__ __device__ inline W
word_in(unsigned long long a, unsigned long long b, int j)
{
    if constexpr (sizeof(W) == 4)
    {
        const unsigned long long x = j < 2 ? a : b;
        return static_cast<W>((j & 1) != 0 ? x >> 32 : x & 0xffffffffull);
    }
    else if constexpr (sizeof(W) == 8)
    {
        return static_cast<W>(j == 0 ? a : b);
    }
    else
    {
        return W{ a, b };
    }
}

// Kernel view of a wide table (trivially copyable, passed by value).
template <typename Key, typename T, typename Hash, typename KeyEqual = void>
struct wide_ref
{
    using key_type = Key;
    using hasher = Hash;
    using key_equal = KeyEqual;
    using W = wide_word_of<Key>;
    using WW = wide_word<W>;
    static constexpr int G = 128 / static_cast<int>(sizeof(W)); // slots per probe group
    static constexpr bool has_values = wide_mapped_store<T>::stored;
    static constexpr bool has_specials = sizeof(Key) == sizeof(W); // padding keeps shorter keys off the patterns
    using value_store = std::conditional_t<has_values, T, char>;

    W* keys = nullptr;
    value_store* values = nullptr;
    wide_header* hdr = nullptr;
    unsigned int* locks = nullptr; // stripe locks of the device inserts, lock_mask + 1 of them
    std::int64_t lock_mask = 0;
    std::int64_t max_size = 0;
    std::int64_t num_groups = 0;
    std::int64_t bucket_count = 0;
    int bucket_bits = 0;

    __host__ __device__ std::int64_t
    special_base() const
    {
        return num_groups * G;
    }

    // one past the last slot (the two out-of-band slots included): end()
    __host__ __device__ std::int64_t
    end_slot() const
    {
        return num_groups * G + 2;
    }

    __host__ __device__ std::int64_t
    home(std::uint64_t hash) const
    {
        return sg::detail::group_of_bucket(sg::detail::fibonacci_bucket(hash, bucket_bits), bucket_bits, num_groups);
    }

    // Whether stored key word x holds a key equal to the key of word w.
    __host__ __device__ static bool
    same(const W& x, const W& w)
    {
        if constexpr (std::is_void<KeyEqual>::value)
        {
            return x == w;
        }
        else
        {
            return KeyEqual{}(from_wide<Key>(x), from_wide<Key>(w));
        }
    }

    __host__ __device__ static int
    special_of(const W& w)
    {
        if constexpr (has_specials)
        {
            return w == WW::empty() ? 0 : (w == WW::tomb() ? 1 : -1);
        }
        else
        {
            return -1;
        }
    }

    template <typename Value>
    __host__ __device__ static Key
    key_of(const Value& v)
    {
        if constexpr (std::is_void<T>::value)
        {
            return v;
        }
        else
        {
            return v.first;
        }
    }

    template <typename Value>
    __host__ __device__ static const value_store*
    mapped_of(const Value& v)
    {
        if constexpr (has_values)
        {
            return &v.second;
        }
        else
        {
            return nullptr;
        }
    }

#if defined(__CUDACC__)
    struct group_masks
    {
        unsigned match; // stored keys the predicate accepts
        unsigned free;  // never-used slots
        unsigned tomb;  // erased slots
    };

    // Masks of group g (bit s = slot s of the group); slots at index >= max_size are in none of them.
    template <typename Pred>
    __device__ group_masks
    scan(std::int64_t g, Pred pred) const
    {
        constexpr int per = 16 / static_cast<int>(sizeof(W));
        group_masks m{ 0u, 0u, 0u };
        const char* p = reinterpret_cast<const char*>(keys + g * G);
        const std::int64_t live = max_size - g * G;
#pragma unroll
        for (int c = 0; c < 8; ++c)
        {
            unsigned long long a, b;
            asm volatile("ld.global.cg.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p + 16 * c) : "memory");
#pragma unroll
            for (int j = 0; j < per; ++j)
            {
                const int s = c * per + j;
                if (s >= live)
                {
                    continue;
                }
                const W w = word_in<W>(a, b, j);
                const unsigned bit = 1u << s;
                if (w == WW::empty())
                {
                    m.free |= bit;
                }
                else if (w == WW::tomb())
                {
                    m.tomb |= bit;
                }
                else if (pred(w))
                {
                    m.match |= bit;
                }
            }
        }
        return m;
    }

    __device__ unsigned
    special_state(int s) const
    {
        return *static_cast<volatile unsigned*>(&hdr->special_state[s]);
    }

    // First slot along the key's probe chain whose stored key the predicate accepts, or -1.
    template <typename Pred>
    __device__ std::int64_t
    find_if(std::uint64_t hash, Pred pred) const
    {
        std::int64_t g = home(hash);
        for (std::int64_t n = 0; n < num_groups; ++n)
        {
            const group_masks m = scan(g, pred);
            if (m.match != 0u)
            {
                return g * G + (__ffs(m.match) - 1);
            }
            if (m.free != 0u)
            {
                return -1;
            }
            g = g + 1 == num_groups ? 0 : g + 1;
        }
        return -1;
    }

    // Broadcast of a key word from lane src (full warp).
    __device__ static W
    shfl_word(const W& w, int src)
    {
        if constexpr (sizeof(W) == 16)
        {
            return W{ __shfl_sync(0xffffffffu, w.lo, src), __shfl_sync(0xffffffffu, w.hi, src) };
        }
        else
        {
            return __shfl_sync(0xffffffffu, w, src);
        }
    }

    // The home group of each key of a whole warp that calls together (one key per thread, the shape of a
    // caller's kernel and of the bulk kernels), read as one 128-byte request per key -- 4 lanes taking 32
    // bytes each -- instead of each thread issuing eight 16-byte loads per group.  For this lane's key: the
    // slot holding it (or -1), the group's first never-used and first erased slot (or -1).  The caller makes
    // sure the whole warp is converged (every lane calls).
    struct home_view
    {
        std::int64_t match, first_free, first_tomb;
    };

    __device__ home_view
    warp_home_scan(const W& w, std::int64_t my_home) const
    {
        constexpr int WPS = 32 / static_cast<int>(sizeof(W)); // words per 32-byte sector
        unsigned lane;
        asm("mov.u32 %0, %%laneid;" : "=r"(lane));
        const int tbase = static_cast<int>(lane & ~3u);
        const int q = static_cast<int>(lane & 3u);
        long long hr[4];
        unsigned long long d[4][4];
#pragma unroll
        for (int r = 0; r < 4; ++r)
        {
            hr[r] = __shfl_sync(0xffffffffu, static_cast<long long>(my_home), tbase + r);
            const char* p = reinterpret_cast<const char*>(keys + hr[r] * G) + 32 * q;
            asm volatile("ld.global.cg.v4.u64 {%0,%1,%2,%3}, [%4];"
                         : "=l"(d[r][0]), "=l"(d[r][1]), "=l"(d[r][2]), "=l"(d[r][3])
                         : "l"(p));
        }
        home_view out{ -1, -1, -1 };
#pragma unroll
        for (int r = 0; r < 4; ++r)
        {
            const W wr = shfl_word(w, tbase + r);
            const std::int64_t first = hr[r] * G + q * WPS;
            unsigned mm = 0u, me = 0u, mt = 0u;
#pragma unroll
            for (int j = 0; j < WPS; ++j)
            {
                // word j of the sector: 16-byte load pair j / (WPS / 2), word j % (WPS / 2) of it
                constexpr int per = WPS / 2;
                const W x = word_in<W>(d[r][2 * (j / per)], d[r][2 * (j / per) + 1], j % per);
                const bool live = first + j < max_size;
                const bool empty = x == WW::empty(), tomb = x == WW::tomb();
                mm |= static_cast<unsigned>(live && !empty && !tomb && same(x, wr)) << j;
                me |= static_cast<unsigned>(live && empty) << j;
                mt |= static_cast<unsigned>(live && tomb) << j;
            }
            const unsigned tm = (__ballot_sync(0xffffffffu, mm != 0u) >> tbase) & 0xFu;
            const unsigned te = (__ballot_sync(0xffffffffu, me != 0u) >> tbase) & 0xFu;
            const unsigned tt = (__ballot_sync(0xffffffffu, mt != 0u) >> tbase) & 0xFu;
            const int om_l = tm != 0u ? __ffs(tm) - 1 : 0;
            const int oe_l = te != 0u ? __ffs(te) - 1 : 0;
            const int ot_l = tt != 0u ? __ffs(tt) - 1 : 0;
            const unsigned om = __shfl_sync(0xffffffffu, mm, tbase + om_l);
            const unsigned oe = __shfl_sync(0xffffffffu, me, tbase + oe_l);
            const unsigned ot = __shfl_sync(0xffffffffu, mt, tbase + ot_l);
            if (q == r)
            {
                const std::int64_t g0 = hr[r] * G;
                out.match = tm != 0u ? g0 + om_l * WPS + (__ffs(om) - 1) : -1;
                out.first_free = te != 0u ? g0 + oe_l * WPS + (__ffs(oe) - 1) : -1;
                out.first_tomb = tt != 0u ? g0 + ot_l * WPS + (__ffs(ot) - 1) : -1;
            }
        }
        return out;
    }

    // find_word for the keys of a whole warp that calls together (warp_home_scan); a key not decided in its
    // home group, an out-of-band key, and the lanes of a partial warp go on alone.
    __device__ std::int64_t
    find_word_warp(const W& w, std::uint64_t hash) const
    {
        if (__activemask() != 0xffffffffu)
        {
            return find_word(w, hash);
        }
        const bool probe = special_of(w) < 0;
        const std::int64_t my_home = probe ? home(hash) : 0;
        const home_view h = warp_home_scan(w, my_home);
        if (!probe)
        {
            return find_word(w, hash);
        }
        if (h.match >= 0 || h.first_free >= 0)
        {
            return h.match;
        }
        // the home group is full of other keys: the rest of the chain alone
        std::int64_t g = my_home + 1 == num_groups ? 0 : my_home + 1;
        for (std::int64_t n = 1; n < num_groups; ++n)
        {
            const group_masks m = scan(g, [&](const W& x) { return same(x, w); });
            if (m.match != 0u)
            {
                return g * G + (__ffs(m.match) - 1);
            }
            if (m.free != 0u)
            {
                return -1;
            }
            g = g + 1 == num_groups ? 0 : g + 1;
        }
        return -1;
    }

    // A bulk insert's first try for the keys of a whole warp (insert-only launch: free slots only disappear):
    // present in the home group, or one claim of the home group's first erased slot (reuse_tombs) or first
    // never-used slot when the group has a never-used slot -- the slot the per-thread insert_word would pick.
    // {-2, false} when the key needs insert_word (claim lost, home group full, out-of-band key, partial warp).
    __device__ wide_insert_result
    insert_word_warp_try(const W& w, std::uint64_t hash, bool reuse_tombs, const value_store* mapped) const
    {
        if (__activemask() != 0xffffffffu)
        {
            return { -2, false };
        }
        const bool probe = special_of(w) < 0;
        const std::int64_t my_home = probe ? home(hash) : 0;
        const home_view h = warp_home_scan(w, my_home);
        if (!probe)
        {
            return { -2, false };
        }
        if (h.match >= 0)
        {
            return { h.match, false };
        }
        if (h.first_free < 0)
        {
            return { -2, false };
        }
        const bool take_tomb = reuse_tombs && h.first_tomb >= 0;
        const std::int64_t slot = take_tomb ? h.first_tomb : h.first_free;
        const W expected = take_tomb ? WW::tomb() : WW::empty();
        const W old = WW::cas(keys + slot, expected, w);
        if (old == expected)
        {
            construct(slot, mapped);
            return { slot, true };
        }
        if (old != WW::empty() && old != WW::tomb() && same(old, w))
        {
            return { slot, false };
        }
        return { -2, false };
    }

    __device__ std::int64_t
    find_word(const W& w, std::uint64_t hash) const
    {
        const int sp = special_of(w);
        if (sp >= 0)
        {
            return special_state(sp) == 1u ? special_base() + sp : -1;
        }
        return find_if(hash, [&](const W& x) { return same(x, w); });
    }

    // Whether stored Key k equals heterogeneous key kl: KeyEqual where it takes the pair (a transparent
    // KeyEqual), else operator==.
    template <typename KeyLike>
    __host__ __device__ static bool
    same_like(const Key& k, const KeyLike& kl)
    {
        if constexpr (!std::is_void<KeyEqual>::value && std::is_invocable<KeyEqual, const Key&, const KeyLike&>::value)
        {
            return KeyEqual{}(k, kl);
        }
        else
        {
            return k == kl;
        }
    }

    // Heterogeneous lookup: a value equal to the stored Key, hashed like it.
    template <typename KeyLike>
    __device__ std::int64_t
    find_like(const KeyLike& k, std::uint64_t hash) const
    {
        if constexpr (has_specials)
        {
            for (int s = 0; s < 2; ++s)
            {
                if (special_state(s) == 1u && same_like(from_wide<Key>(s == 0 ? WW::empty() : WW::tomb()), k))
                {
                    return special_base() + s;
                }
            }
        }
        return find_if(hash, [&](const W& x) { return same_like(from_wide<Key>(x), k); });
    }

    __device__ void
    construct(std::int64_t slot, const value_store* mapped) const
    {
        if constexpr (has_values)
        {
            if (mapped != nullptr)
            {
                new (values + slot) T(*mapped);
            }
        }
    }

    __device__ void
    destroy(std::int64_t slot) const
    {
        if constexpr (has_values && !std::is_trivially_destructible<T>::value)
        {
            values[slot].~T();
        }
    }

    // Out-of-band key s: 0 -> 2 (busy) -> 1 (present) on insert, 1 -> 2 -> 0 on erase.
    __device__ wide_insert_result
    special_insert(int s, const value_store* mapped) const
    {
        const unsigned old = atomicCAS(&hdr->special_state[s], 0u, 2u);
        const std::int64_t slot = special_base() + s;
        if (old != 0u)
        {
            return { slot, false };
        }
        construct(slot, mapped);
        keys[slot] = s == 0 ? WW::empty() : WW::tomb();
        __threadfence();
        atomicExch(&hdr->special_state[s], 1u);
        return { slot, true };
    }

    // Insert of key word w (try_insert, src/stdgpu/impl/unordered_base_detail.cuh:708-809): present ->
    // its slot; else a claim of the first erased slot (bulk inserts, reuse_tombs) or never-used slot of the
    // first group of the probe chain that has a never-used slot.  The caller counts the insert.
    __device__ wide_insert_result
    insert_word(const W& w, std::uint64_t hash, bool reuse_tombs, const value_store* mapped) const
    {
        const int sp = special_of(w);
        if (sp >= 0)
        {
            return special_insert(sp, mapped);
        }
        for (int attempt = 0; attempt < kWideRetry; ++attempt)
        {
            std::int64_t g = home(hash);
            std::int64_t first_tomb = -1; // the chain's first erased slot, for a table without never-used slots
            for (std::int64_t n = 0; n < num_groups; ++n)
            {
                for (int tries = 0;; ++tries)
                {
                    const group_masks m = scan(g, [&](const W& x) { return same(x, w); });
                    if (m.match != 0u)
                    {
                        return { g * G + (__ffs(m.match) - 1), false };
                    }
                    if (m.free == 0u)
                    {
                        if (first_tomb < 0 && m.tomb != 0u)
                        {
                            first_tomb = g * G + (__ffs(m.tomb) - 1);
                        }
                        break; // the chain goes on
                    }
                    if (tries >= kWideRetry)
                    {
                        atomicOr(&hdr->error, sg::detail::kErrRetry);
                        return { -1, false };
                    }
                    const bool take_tomb = reuse_tombs && m.tomb != 0u;
                    const std::int64_t slot = g * G + (__ffs(take_tomb ? m.tomb : m.free) - 1);
                    const W expected = take_tomb ? WW::tomb() : WW::empty();
                    const W old = WW::cas(keys + slot, expected, w);
                    if (old == expected)
                    {
                        construct(slot, mapped);
                        return { slot, true };
                    }
                    if (old != WW::empty() && old != WW::tomb() && same(old, w))
                    {
                        return { slot, false };
                    }
                    // another key took the slot: read the group again
                }
                g = g + 1 == num_groups ? 0 : g + 1;
            }
            // no never-used slot left anywhere: the chain's first erased slot (every slot was read, so the key
            // is absent), else refused
            if (!reuse_tombs || first_tomb < 0)
            {
                return { -1, false };
            }
            const W old = WW::cas(keys + first_tomb, WW::tomb(), w);
            if (old == WW::tomb())
            {
                construct(first_tomb, mapped);
                return { first_tomb, true };
            }
            if (old != WW::empty() && same(old, w))
            {
                return { first_tomb, false };
            }
            // another key took that slot meanwhile: read the chain again
        }
        atomicOr(&hdr->error, sg::detail::kErrRetry);
        return { -1, false };
    }

    // Device insert (insert / emplace, unordered_base_detail.cuh:958-994) under the stripe lock of the key's
    // home group: erased slots are reused beside device erases.  A key found present without the lock, or
    // stored by another thread while this one waits, decides the call without it.
    __device__ wide_insert_result
    insert_word_locked(const W& w, std::uint64_t hash, const value_store* mapped) const
    {
        if (special_of(w) >= 0 || locks == nullptr)
        {
            return insert_word(w, hash, false, mapped);
        }
        std::int64_t slot = find_word_warp(w, hash);
        if (slot >= 0)
        {
            return { slot, false };
        }
        unsigned int* l = locks + (static_cast<std::uint64_t>(home(hash)) & static_cast<std::uint64_t>(lock_mask));
        unsigned int backoff = 32;
        for (long long polls = 0; polls < sg::detail::kWaitLimit; ++polls)
        {
            if (*reinterpret_cast<volatile unsigned int*>(l) == 0u && atomicCAS(l, 0u, 1u) == 0u)
            {
                sg::detail::fence_acq_rel_gpu();
                const wide_insert_result r = insert_word(w, hash, true, mapped);
                sg::detail::fence_acq_rel_gpu();
                atomicExch(l, 0u);
                return r;
            }
            if ((polls & 15) == 15 && (slot = find_word(w, hash)) >= 0)
            {
                return { slot, false };
            }
            __nanosleep(backoff);
            backoff = backoff < 256 ? backoff * 2 : 256;
        }
        atomicOr(&hdr->error, sg::detail::kErrRetry);
        return { -1, false };
    }

    // Erase of key word w (try_erase, src/stdgpu/impl/unordered_base_detail.cuh:811-913); the caller counts it.
    __device__ bool
    erase_word(const W& w, std::uint64_t hash) const
    {
        const int sp = special_of(w);
        if (sp >= 0)
        {
            if (atomicCAS(&hdr->special_state[sp], 1u, 2u) != 1u)
            {
                return false;
            }
            destroy(special_base() + sp);
            __threadfence();
            atomicExch(&hdr->special_state[sp], 0u);
            return true;
        }
        const std::int64_t slot = find_word_warp(w, hash);
        if (slot < 0)
        {
            return false;
        }
        // the word found there: the key's own bytes, or an equal key's
        const W stored = std::is_void<KeyEqual>::value ? w : WW::load(keys + slot);
        if (stored == WW::empty() || stored == WW::tomb() || !same(stored, w) ||
            WW::cas(keys + slot, stored, WW::tomb()) != stored)
        {
            return false;
        }
        destroy(slot);
        return true;
    }

    // Stored keys whose bucket is b (bucket_size, src/stdgpu/impl/unordered_base_detail.cuh:568-609): they
    // all sit along the chain from b's home group up to its first group with a never-used slot.
    __device__ std::int64_t
    bucket_size(std::int64_t b) const
    {
        const auto bucket_of = [&](const W& x) {
            return static_cast<std::int64_t>(
                    sg::detail::fibonacci_bucket(static_cast<std::uint64_t>(Hash{}(from_wide<Key>(x))), bucket_bits));
        };
        if (b < 0 || b >= bucket_count)
        {
            return 0; // no such bucket (the reference requires b < bucket_count())
        }
        std::int64_t count = 0;
        std::int64_t g = sg::detail::group_of_bucket(static_cast<std::uint64_t>(b), bucket_bits, num_groups);
        for (std::int64_t n = 0; n < num_groups; ++n)
        {
            const group_masks m = scan(g, [&](const W& x) { return bucket_of(x) == b; });
            count += __popc(m.match);
            if (m.free != 0u)
            {
                break;
            }
            g = g + 1 == num_groups ? 0 : g + 1;
        }
        if constexpr (has_specials)
        {
            for (int s = 0; s < 2; ++s)
            {
                count += special_state(s) == 1u && bucket_of(s == 0 ? WW::empty() : WW::tomb()) == b ? 1 : 0;
            }
        }
        return count;
    }
#endif
};

#if defined(__CUDACC__)
// d (+-1) added to a counter by the lanes of the warp that run the call together: one atomic per group of
// converged lanes (device calls of one launch otherwise queue on the counter's address).
__device__ inline void
wide_converged_add(unsigned long long* counter, int d)
{
    const unsigned m = __activemask();
    unsigned lane;
    asm("mov.u32 %0, %%laneid;" : "=r"(lane));
    const int sum = static_cast<int>(__reduce_add_sync(m, static_cast<unsigned>(d)));
    if (lane == static_cast<unsigned>(__ffs(m) - 1) && sum != 0)
    {
        atomicAdd(counter, static_cast<unsigned long long>(static_cast<long long>(sum)));
    }
}

// One warp's sum of per-lane deltas added to a counter (every lane of a full warp calls it).
__device__ inline void
wide_flush(unsigned long long* counter, long long delta)
{
    for (int off = 16; off > 0; off >>= 1)
    {
        delta += __shfl_down_sync(0xffffffffu, delta, off);
    }
    if ((threadIdx.x & 31u) == 0u && delta != 0)
    {
        atomicAdd(counter, static_cast<unsigned long long>(delta));
    }
}

// Bulk insert over value_type elements (insert(begin, end), unordered_base_detail.cuh:470-495, :996-1017).
template <typename Ref, typename Value>
__global__ void
k_wide_insert(Ref t, const Value* in, std::int64_t n)
{
    using Key = typename Ref::key_type;
    long long added = 0;
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    for (std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        const Value& v = in[i];
        const Key key = Ref::key_of(v);
        const typename Ref::W w = to_wide<typename Ref::W>(key);
        const std::uint64_t h = static_cast<std::uint64_t>(typename Ref::hasher{}(key));
        wide_insert_result r = t.insert_word_warp_try(w, h, true, Ref::mapped_of(v));
        if (r.slot == -2)
        {
            r = t.insert_word(w, h, true, Ref::mapped_of(v));
        }
        added += r.inserted ? 1 : 0;
    }
    wide_flush(&t.hdr->size, added);
}

// Bulk erase over keys (erase(begin, end), unordered_base_detail.cuh:497-522, :1045-1066).
template <typename Ref>
__global__ void
k_wide_erase(Ref t, const typename Ref::key_type* in, std::int64_t n)
{
    using Key = typename Ref::key_type;
    long long removed = 0;
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    for (std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        const Key key = in[i];
        removed += t.erase_word(to_wide<typename Ref::W>(key), static_cast<std::uint64_t>(typename Ref::hasher{}(key)))
                           ? 1
                           : 0;
    }
    wide_flush(&t.hdr->size, -removed);
}

// valid() (unordered_base_detail.cuh:1194-1218): probe words past max_size never used, every stored key
// found again through its own hash at its own slot (so it is reachable and stored once), out-of-band states
// settled, and the stored count (out-of-band keys included) in hdr->count for the caller to compare.
template <typename Ref>
__global__ void
k_wide_valid(Ref t)
{
    using W = typename Ref::W;
    using WW = typename Ref::WW;
    using Key = typename Ref::key_type;
    long long count = 0;
    bool bad = false;
    const std::int64_t total = t.num_groups * Ref::G;
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    for (std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x; i < total; i += stride)
    {
        const W w = t.keys[i];
        if (w == WW::empty())
        {
            continue;
        }
        if (i >= t.max_size)
        {
            bad = true;
            continue;
        }
        if (w == WW::tomb())
        {
            continue;
        }
        ++count;
        bad = bad || t.find_word(w, static_cast<std::uint64_t>(typename Ref::hasher{}(from_wide<Key>(w)))) != i;
    }
    if (blockIdx.x == 0 && threadIdx.x < 2)
    {
        const unsigned s = t.hdr->special_state[threadIdx.x];
        bad = bad || s > 1u || (s == 1u && !Ref::has_specials);
        count += s == 1u ? 1 : 0;
    }
    wide_flush(&t.hdr->count, count);
    if (bad)
    {
        atomicOr(&t.hdr->bad, 1u);
    }
}

// device_range() (unordered_base_detail.cuh:136-208): the slot indices of the stored elements; a warp
// takes 32 consecutive slots and reserves its run with one atomic, so the order between runs is arbitrary,
// as in the reference.
template <typename Ref>
__global__ void
k_wide_range(Ref t, std::int32_t* out)
{
    using W = typename Ref::W;
    using WW = typename Ref::WW;
    const std::int64_t total = t.num_groups * Ref::G;
    const unsigned lane = threadIdx.x & 31u;
    const std::int64_t warp = (blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x) >> 5;
    const std::int64_t warps = (static_cast<std::int64_t>(gridDim.x) * blockDim.x) >> 5;
    for (std::int64_t base = warp * 32; base < total; base += warps * 32)
    {
        const std::int64_t i = base + lane;
        bool stored = false;
        if (i < total && i < t.max_size)
        {
            const W w = t.keys[i];
            stored = w != WW::empty() && w != WW::tomb();
        }
        const unsigned ball = __ballot_sync(0xffffffffu, stored);
        unsigned long long pos = 0;
        if (lane == 0u && ball != 0u)
        {
            pos = atomicAdd(&t.hdr->count, static_cast<unsigned long long>(__popc(ball)));
        }
        pos = __shfl_sync(0xffffffffu, pos, 0);
        if (stored)
        {
            out[pos + __popc(ball & ((1u << lane) - 1u))] = static_cast<std::int32_t>(i);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < 2 && t.hdr->special_state[threadIdx.x] == 1u)
    {
        out[atomicAdd(&t.hdr->count, 1ull)] = static_cast<std::int32_t>(t.special_base() + threadIdx.x);
    }
}

// clear() / destroyDeviceObject() of a mapped type with a destructor: destroy_values
// (unordered_base_detail.cuh:1238-1243, :1318-1321) over the stored elements.
template <typename Ref>
__global__ void
k_wide_destroy(Ref t)
{
    using W = typename Ref::W;
    using WW = typename Ref::WW;
    const std::int64_t total = t.num_groups * Ref::G;
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    for (std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x; i < total; i += stride)
    {
        const W w = t.keys[i];
        if (i < t.max_size && w != WW::empty() && w != WW::tomb())
        {
            t.destroy(i);
        }
    }
    if (blockIdx.x == 0 && threadIdx.x < 2 && t.hdr->special_state[threadIdx.x] == 1u)
    {
        t.destroy(t.special_base() + threadIdx.x);
    }
}
#endif


// Iterator of find(): a slot; dereferencing gives its element as a value_type copy.
template <typename Ref, typename T, typename Value>
struct wide_iterator
{
    const typename Ref::W* key = nullptr;
    const typename Ref::value_store* val = nullptr;

#if defined(__CUDACC__)
    __device__ Value
    operator*() const
    {
        using Key = typename Ref::key_type;
        const Key k = from_wide<Key>(*key);
        if constexpr (std::is_void<T>::value)
        {
            return k;
        }
        else if constexpr (Ref::has_values)
        {
            return Value(k, *val);
        }
        else
        {
            return Value(k, T{});
        }
    }

    struct arrow
    {
        Value v;
        __device__ const Value*
        operator->() const
        {
            return &v;
        }
    };

    __device__ arrow
    operator->() const
    {
        return arrow{ **this };
    }
#endif

    __host__ __device__ bool
    operator==(const wide_iterator& o) const
    {
        return key == o.key;
    }

    __host__ __device__ bool
    operator!=(const wide_iterator& o) const
    {
        return key != o.key;
    }
};

// device_range() of a wide table: the stored elements through their slot indices.
template <typename Ref, typename T>
struct wide_range
{
    const std::int32_t* indices = nullptr;
    index_t count = 0;
    Ref table{};

    __host__ __device__ index_t
    size() const
    {
        return count;
    }

#if defined(__CUDACC__)
    __device__ typename Ref::key_type
    key(index_t i) const
    {
        return from_wide<typename Ref::key_type>(table.keys[indices[i]]);
    }

    template <typename U = T, typename = std::enable_if_t<!std::is_void<U>::value>>
    __device__ U
    mapped(index_t i) const
    {
        if constexpr (Ref::has_values)
        {
            return table.values[indices[i]];
        }
        else
        {
            return U{};
        }
    }
#endif
};

template <typename P>
inline bool
wide_alloc(P** p, std::size_t bytes)
{
    return cudaMalloc(reinterpret_cast<void**>(p), bytes > 0 ? bytes : 1) == cudaSuccess;
}

template <typename Key, typename T, typename Hash, typename Value, typename Derived, typename KeyEqual = void>
class wide_unordered
{
    static_assert(sizeof(Key) <= 16, "a key type of at most 16 bytes");

public:
    using ref_type = wide_ref<Key, T, Hash, KeyEqual>;
    using W = typename ref_type::W;
    using value_store = typename ref_type::value_store;
    using key_type = Key;
    using value_type = Value;
    using hasher = Hash;
    using iterator = wide_iterator<ref_type, T, Value>;
    using const_iterator = iterator;

    // createDeviceObject(capacity): the reference's geometry (unordered_base_detail.cuh:1254-1308)
    static Derived
    createDeviceObject(const index_t& capacity)
    {
        return createDeviceObject(execution::device, capacity);
    }

    static Derived
    createDeviceObject(execution::device_policy policy, const index_t& capacity)
    {
        return create_impl(policy, capacity, sg_allocator{});
    }

    // createDeviceObject(capacity, allocator): every device block of the object from `alloc`
    static Derived
    create_with_allocator(execution::device_policy policy, const index_t& capacity, const sg_allocator& alloc)
    {
        return create_impl(policy, capacity, alloc);
    }

    static Derived
    create_impl(execution::device_policy policy, const index_t& capacity, const sg_allocator& alloc)
    {
        sg_geometry geo{};
        const sg_status gst = sg_unordered_geometry_for(SG_SET_U32, capacity, &geo);
        if (gst != SG_OK && alloc.release_ctx != nullptr)
        {
            alloc.release_ctx(alloc.ctx);
        }
        gb300_check(gst, "createDeviceObject");
        Derived d;
        d._alloc = alloc;
        ref_type& t = d._t;
        t.max_size = geo.max_size;
        t.bucket_count = geo.bucket_count;
        t.num_groups = (geo.max_size + ref_type::G - 1) / ref_type::G;
        while ((std::int64_t{ 1 } << t.bucket_bits) < geo.bucket_count)
        {
            ++t.bucket_bits;
        }
        const std::int64_t slots = t.end_slot();
        std::int64_t nlocks = 256; // one per 16 probe groups, a power of two in [256, 2^22]
        while (nlocks < t.num_groups / 16 && nlocks < (std::int64_t{ 1 } << 22))
        {
            nlocks <<= 1;
        }
        t.lock_mask = nlocks - 1;
        bool ok = d.block(&t.keys, sizeof(W) * slots) && d.block(&t.hdr, sizeof(wide_header)) &&
                  d.block(&d._range, sizeof(std::int32_t) * (geo.max_size + 2)) &&
                  d.block(&t.locks, sizeof(unsigned int) * nlocks);
        if (ok && ref_type::has_values)
        {
            ok = d.block(&t.values, sizeof(value_store) * slots);
        }
        if (!ok)
        {
            free_all(d);
            gb300_check(SG_ERR_OOM, "createDeviceObject");
            return d;
        }
        const bool set = cudaMemsetAsync(t.keys, 0xff, sizeof(W) * slots, policy.stream) == cudaSuccess &&
                         cudaMemsetAsync(t.hdr, 0, sizeof(wide_header), policy.stream) == cudaSuccess &&
                         cudaMemsetAsync(t.locks, 0, sizeof(unsigned int) * nlocks, policy.stream) == cudaSuccess &&
                         cudaStreamSynchronize(policy.stream) == cudaSuccess;
        gb300_check(set ? SG_OK : SG_ERR_CUDA, "createDeviceObject");
        return d;
    }

    // destroyDeviceObject (unordered_base_detail.cuh:1310-1348): a mapped type with a destructor is cleared
    // first, so every stored object is destroyed.
    static void
    destroyDeviceObject(Derived& d)
    {
        destroyDeviceObject(execution::device, d);
    }

    static void
    destroyDeviceObject(execution::device_policy policy, Derived& d)
    {
        if (d._t.keys != nullptr && destroys_values())
        {
            d.clear(policy);
        }
        cudaStreamSynchronize(policy.stream);
        free_all(d);
    }

    void
    insert(const value_type* begin, const value_type* end)
    {
        insert(execution::device, begin, end);
    }

    void
    insert(execution::device_policy policy, const value_type* begin, const value_type* end)
    {
        const std::int64_t n = end - begin;
        if (n <= 0)
        {
            return;
        }
        k_wide_insert<ref_type, value_type><<<grid_of(n), 256, 0, policy.stream>>>(_t, begin, n);
        gb300_check(cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA, "insert");
    }

    void
    erase(const key_type* begin, const key_type* end)
    {
        erase(execution::device, begin, end);
    }

    void
    erase(execution::device_policy policy, const key_type* begin, const key_type* end)
    {
        const std::int64_t n = end - begin;
        if (n <= 0)
        {
            return;
        }
        k_wide_erase<ref_type><<<grid_of(n), 256, 0, policy.stream>>>(_t, begin, n);
        gb300_check(cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA, "erase");
    }

    index_t
    size(execution::device_policy policy = execution::device) const
    {
        return _t.keys == nullptr ? 0 : static_cast<index_t>(header(policy).size); // default-constructed: empty
    }

    bool
    empty(execution::device_policy policy = execution::device) const
    {
        return size(policy) == 0;
    }

    bool
    full(execution::device_policy policy = execution::device) const
    {
        return size(policy) == max_size();
    }

    __host__ __device__ index_t
    max_size() const noexcept
    {
        return static_cast<index_t>(_t.max_size);
    }

    __host__ __device__ index_t
    bucket_count() const
    {
        return static_cast<index_t>(_t.bucket_count);
    }

    float
    load_factor(execution::device_policy policy = execution::device) const
    {
        return static_cast<float>(size(policy)) / static_cast<float>(bucket_count());
    }

    __host__ __device__ float
    max_load_factor() const
    {
        return 1.0F;
    }

    // clear() (unordered_base_detail.cuh:1220-1252): stored objects destroyed, every slot never used again
    void
    clear(execution::device_policy policy = execution::device)
    {
        if (destroys_values())
        {
            k_wide_destroy<ref_type><<<grid_of(_t.num_groups * ref_type::G), 256, 0, policy.stream>>>(_t);
        }
        const bool ok = cudaGetLastError() == cudaSuccess &&
                        cudaMemsetAsync(_t.keys, 0xff, sizeof(W) * _t.end_slot(), policy.stream) == cudaSuccess &&
                        cudaMemsetAsync(_t.hdr, 0, sizeof(wide_header), policy.stream) == cudaSuccess;
        gb300_check(ok ? SG_OK : SG_ERR_CUDA, "clear");
    }

    // valid(): structure, reachability and uniqueness of every stored key, the stored count against size(),
    // and no call that gave up (unordered_base_detail.cuh:1192-1218)
    bool
    valid(execution::device_policy policy = execution::device) const
    {
        if (_t.keys == nullptr)
        {
            return true;
        }
        bool ok = cudaMemsetAsync(&_t.hdr->bad, 0, sizeof(unsigned int), policy.stream) == cudaSuccess &&
                  cudaMemsetAsync(&_t.hdr->count, 0, sizeof(unsigned long long), policy.stream) == cudaSuccess;
        k_wide_valid<ref_type><<<grid_of(_t.num_groups * ref_type::G), 256, 0, policy.stream>>>(_t);
        ok = ok && cudaGetLastError() == cudaSuccess;
        gb300_check(ok ? SG_OK : SG_ERR_CUDA, "valid");
        const wide_header h = header(policy);
        return h.bad == 0u && h.error == 0u && h.count == h.size;
    }

    wide_range<ref_type, T>
    device_range(execution::device_policy policy = execution::device)
    {
        bool ok = cudaMemsetAsync(&_t.hdr->count, 0, sizeof(unsigned long long), policy.stream) == cudaSuccess;
        k_wide_range<ref_type><<<grid_of(_t.num_groups * ref_type::G), 256, 0, policy.stream>>>(_t, _range);
        ok = ok && cudaGetLastError() == cudaSuccess;
        gb300_check(ok ? SG_OK : SG_ERR_CUDA, "device_range");
        return wide_range<ref_type, T>{ _range, static_cast<index_t>(header(policy).count), _t };
    }

    // bucket(key): the fibonacci hashing of Hash(key) (unordered_base_detail.cuh:547-564)
    __host__ __device__ index_t
    bucket(const key_type& key) const
    {
        return static_cast<index_t>(
                sg::detail::fibonacci_bucket(static_cast<std::uint64_t>(Hash{}(key)), _t.bucket_bits));
    }

    __host__ __device__ bool
    is_null() const
    {
        return _t.keys == nullptr;
    }

#if defined(__CUDACC__)
    // ---- device members
    __device__ iterator
    end() const
    {
        return iterator{ _t.keys + _t.end_slot(), nullptr };
    }

    __device__ index_t
    bucket_size(index_t n) const
    {
        return static_cast<index_t>(_t.bucket_size(n));
    }

    __device__ iterator
    find(const key_type& key) const
    {
        return at(_t.find_word_warp(to_wide<W>(key), static_cast<std::uint64_t>(Hash{}(key))));
    }

    __device__ bool
    contains(const key_type& key) const
    {
        return find(key) != end();
    }

    __device__ index_t
    count(const key_type& key) const
    {
        return contains(key) ? 1 : 0;
    }

    // Heterogeneous lookups (src/stdgpu/impl/unordered_base.cuh:241-298) with a transparent Hash.
    template <typename KeyLike, typename H = Hash, typename = typename H::is_transparent,
              typename = std::enable_if_t<!std::is_same<KeyLike, Key>::value>>
    __device__ iterator
    find(const KeyLike& k) const
    {
        return at(_t.find_like(k, static_cast<std::uint64_t>(Hash{}(k))));
    }

    template <typename KeyLike, typename H = Hash, typename = typename H::is_transparent,
              typename = std::enable_if_t<!std::is_same<KeyLike, Key>::value>>
    __device__ bool
    contains(const KeyLike& k) const
    {
        return find(k) != end();
    }

    template <typename KeyLike, typename H = Hash, typename = typename H::is_transparent,
              typename = std::enable_if_t<!std::is_same<KeyLike, Key>::value>>
    __device__ index_t
    count(const KeyLike& k) const
    {
        return contains(k) ? 1 : 0;
    }

    // erase(key) (unordered_base_detail.cuh:1019-1043)
    __device__ index_t
    erase(const key_type& key) const
    {
        if (!_t.erase_word(to_wide<W>(key), static_cast<std::uint64_t>(Hash{}(key))))
        {
            return 0;
        }
        wide_converged_add(&_t.hdr->size, -1);
        return 1;
    }
#endif

protected:
    static constexpr bool
    destroys_values()
    {
        return ref_type::has_values && !std::is_trivially_destructible<value_store>::value;
    }

    // a device block of this object: its own allocator's, else cudaMalloc
    template <typename P>
    bool
    block(P** p, std::size_t bytes)
    {
        if (_alloc.alloc != nullptr)
        {
            *p = own_alloc<P>(_alloc, bytes);
            return *p != nullptr;
        }
        return wide_alloc(p, bytes);
    }

    void
    unblock(void* p)
    {
        if (p == nullptr)
        {
            return;
        }
        if (_alloc.alloc != nullptr)
        {
            _alloc.release(p, _alloc.ctx);
        }
        else
        {
            cudaFree(p);
        }
    }

    // frees every block and drops the allocator's context
    static void
    free_all(Derived& d)
    {
        if (d._alloc.alloc != nullptr)
        {
            cudaDeviceSynchronize(); // as cudaFree does, before the allocator may hand the memory on
        }
        d.unblock(d._t.keys);
        d.unblock(d._t.values);
        d.unblock(d._t.hdr);
        d.unblock(d._range);
        d.unblock(d._t.locks);
        if (d._alloc.release_ctx != nullptr)
        {
            d._alloc.release_ctx(d._alloc.ctx);
        }
        d._t = ref_type{};
        d._range = nullptr;
        d._alloc = sg_allocator{};
    }

    wide_header
    header(execution::device_policy policy) const
    {
        wide_header h{};
        const bool ok = cudaMemcpyAsync(&h, _t.hdr, sizeof(h), cudaMemcpyDeviceToHost, policy.stream) == cudaSuccess &&
                        cudaStreamSynchronize(policy.stream) == cudaSuccess;
        gb300_check(ok ? SG_OK : SG_ERR_CUDA, "size");
        return h;
    }

#if defined(__CUDACC__)
    __device__ iterator
    at(std::int64_t slot) const
    {
        if (slot < 0)
        {
            return end();
        }
        return iterator{ _t.keys + slot, ref_type::has_values ? _t.values + slot : nullptr };
    }

    // insert(value) / emplace (unordered_base_detail.cuh:958-994) under the key's stripe lock, so erased
    // slots are reused beside device erases
    __device__ pair<iterator, bool>
    insert_impl(const key_type& key, const value_store* mapped) const
    {
        const wide_insert_result r =
                _t.insert_word_locked(to_wide<W>(key), static_cast<std::uint64_t>(Hash{}(key)), mapped);
        if (!r.inserted)
        {
            return pair<iterator, bool>(end(), false);
        }
        wide_converged_add(&_t.hdr->size, 1);
        return pair<iterator, bool>(at(r.slot), true);
    }
#endif

    ref_type _t{};
    std::int32_t* _range = nullptr;
    sg_allocator _alloc{}; // the object's own allocator (createDeviceObject(capacity, allocator)), or none
};

template <typename Key, typename T, typename Hash, typename Derived, typename KeyEqual = void>
class wide_map : public wide_unordered<Key, T, Hash, pair<const Key, T>, Derived, KeyEqual>
{
    using base = wide_unordered<Key, T, Hash, pair<const Key, T>, Derived, KeyEqual>;

public:
    using mapped_type = T;
    using typename base::iterator;
    using typename base::value_type;
    using base::erase;
    using base::insert;

#if defined(__CUDACC__)
    __device__ pair<iterator, bool>
    insert(const value_type& value) const
    {
        return this->insert_impl(value.first, base::ref_type::mapped_of(value));
    }

    __device__ pair<iterator, bool>
    emplace(const Key& key, const T& mapped) const
    {
        return insert(value_type(key, mapped));
    }
#endif
};

template <typename Key, typename Hash, typename Derived, typename KeyEqual = void>
class wide_set : public wide_unordered<Key, void, Hash, Key, Derived, KeyEqual>
{
    using base = wide_unordered<Key, void, Hash, Key, Derived, KeyEqual>;

public:
    using typename base::iterator;
    using typename base::value_type;
    using base::erase;
    using base::insert;

#if defined(__CUDACC__)
    __device__ pair<iterator, bool>
    insert(const value_type& key) const
    {
        return this->insert_impl(key, nullptr);
    }

    __device__ pair<iterator, bool>
    emplace(const Key& key) const
    {
        return insert(key);
    }
#endif
};

} // namespace detail
} // namespace stdgpu

#endif

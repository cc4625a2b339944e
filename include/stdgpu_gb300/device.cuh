// Native device-side calls on a table, for use inside a caller's own kernels
// (the reference's device member functions find / contains / count / insert /
// emplace / erase, src/stdgpu/impl/unordered_base_detail.cuh:619-706, 958-994,
// 1019-1043).  One calling thread per key.  When a whole warp calls together
// (the usual shape: one key per thread), lookups -- and the lock-free scans of
// insert and erase -- read each key's home group as one 128-byte request, four
// lanes taking 32 bytes each; a partial warp, and a key that goes on past its
// home group, read alone.  The header counters (size, erased slots, refusals)
// take one atomic per group of lanes that call together.
//
// Concurrency within one launch:
//  * insert / emplace take the stripe lock of the key's home group (the
//    table's insert_locks; a bounded wait), scan the probe sequence for the
//    key up to the first group holding a never-used slot, and claim the first
//    free slot -- erased or never used -- with a compare-and-swap over the
//    whole slot.  All inserts of one key share the lock, so they never scan and
//    claim at the same time (the lock word carries a version that each release
//    advances: an insert that takes the lock at the version it read before its
//    lock-free scan knows no insert of its stripe finished in between and claims
//    the slot that scan found): a key is stored at most once and exactly one of
//    several concurrent inserts of an absent key reports success, while erases
//    (which take no lock) run in the same launch and free slots that the next
//    inserts reuse -- as the reference's device insert, which locks the bucket
//    (src/stdgpu/impl/unordered_base_detail.cuh:708-809, 958-994).  A view
//    without insert_locks falls back to claiming never-used slots only, which
//    needs no lock.  Device calls and the bulk entry points must not run on a
//    table at the same time.
//  * erase marks the slot erased (compare-and-swap key -> erased marker);
//    exactly one of several concurrent erases of a key reports success.
//  * With the reference's excess-list accounting on (v.bucket_heads), an
//    insert also takes its bucket's own slot or one of the excess slots, and
//    is refused once those run out, as the reference's insert loop refuses it
//    (unordered_base_detail.cuh:980-981); erase then takes the stripe lock
//    too, and gives the bucket's slot or the excess slot back.
//  * insert writes the key and its mapped value with one compare-and-swap over
//    the whole slot (up to 16 bytes), so a concurrent find sees either no key
//    or the key with its value (the reference orders the two with its per-slot
//    lock).
//
// HashFn maps a key word to the 64-bit hash whose fibonacci hashing gives the
// reference bucket (identity for integer keys; a custom key type packs into the
// key word and supplies the reference's Hash, see stdgpu_gb300/stdgpu.cuh).
#ifndef STDGPU_GB300_DEVICE_CUH
#define STDGPU_GB300_DEVICE_CUH

#include <stdint.h>

#include "../stdgpu_gb300.h"
#include "detail/layout.cuh"

namespace sg
{

template <int KIND, class HashFn = detail::identity_word_hash>
struct unordered_ref
{
    using C = detail::kind_consts<KIND>;
    using key_type = typename C::K;
    using mapped_type = typename C::V;
    static constexpr int G = C::slots_per_group;
    static constexpr int SPL = C::slots_per_lane;

    sg_unordered_view v;
    // A bulk kernel's per-thread counts: the header counters' changes accumulate here, to be added once per
    // block, instead of one atomic per key on each counter (nullptr: every call updates the header).
    detail::call_counts* defer = nullptr;

    // d (+-1) added to a header counter by the lanes of the warp that run this call together: one atomic
    // per group of converged lanes instead of one per lane on the same address (the counters' updates are
    // what bounds many device calls of one launch otherwise).
    __device__ __forceinline__ static void
    warp_add(unsigned long long* counter, int d)
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

    __device__ __forceinline__ void
    add_size(int d) const
    {
        if (defer != nullptr)
        {
            defer->size += d;
        }
        else
        {
            warp_add(&header()->size, d);
        }
    }

    __device__ __forceinline__ void
    add_tombs(int d) const
    {
        if (defer != nullptr)
        {
            defer->tombs += d;
        }
        else
        {
            warp_add(&header()->tombstones, d);
        }
    }

    __device__ __forceinline__ void
    add_refused() const
    {
        if (defer != nullptr)
        {
            defer->refused += 1;
        }
        else
        {
            warp_add(&header()->refused, 1);
        }
    }

    __device__ __forceinline__ void
    add_excess(long long d) const
    {
        if (defer != nullptr)
        {
            defer->excess += d;
        }
        else
        {
            atomicAdd(&header()->excess_used, static_cast<unsigned long long>(d));
        }
    }

    __device__ __forceinline__ detail::table_header*
    header() const
    {
        return static_cast<detail::table_header*>(v.header);
    }

    __device__ __forceinline__ char*
    slot_ptr(int64_t slot) const
    {
        return static_cast<char*>(v.slots) + slot * C::slot_bytes;
    }

    __device__ __forceinline__ const uint4*
    group_ptr(int64_t g) const
    {
        return reinterpret_cast<const uint4*>(static_cast<const char*>(v.slots) + g * detail::kGroupBytes);
    }

    // bucket(key): the reference's fibonacci hashing of the key's hash
    __device__ __forceinline__ int64_t
    bucket(key_type key) const
    {
        return static_cast<int64_t>(detail::fibonacci_bucket(HashFn{}(key), v.bucket_bits));
    }

    __device__ __forceinline__ int64_t
    home_group(key_type key) const
    {
        return detail::group_of_bucket(detail::fibonacci_bucket(HashFn{}(key), v.bucket_bits), v.bucket_bits,
                                       v.num_groups);
    }

    __device__ __forceinline__ static bool
    is_special(key_type key)
    {
        return key >= C::tomb_key;
    }

    __device__ __forceinline__ int64_t
    special_slot(key_type key) const
    {
        return v.num_groups * G + (key == C::empty_key ? 0 : 1);
    }

    // Slot index of key, or -1.  Stops at the first group holding a never-used slot.
    __device__ __forceinline__ int64_t
    find_slot(key_type key) const
    {
        return find_slot_warp(key, home_group(key), nullptr);
    }

    // Key and mapped value of sub-slot s of a lane's 32-byte sector w.
    __device__ __forceinline__ static key_type
    sector_key(const uint32_t (&w)[8], int s)
    {
        const int h = s / SPL;
        return detail::key_in_lane<KIND>(make_uint4(w[4 * h], w[4 * h + 1], w[4 * h + 2], w[4 * h + 3]), s % SPL);
    }

    __device__ __forceinline__ static mapped_type
    sector_value(const uint32_t (&w)[8], int s)
    {
        const int h = s / SPL;
        return detail::value_in_lane<KIND>(make_uint4(w[4 * h], w[4 * h + 1], w[4 * h + 2], w[4 * h + 3]), s % SPL);
    }

    // find_slot (and, with out, the mapped value) for the keys of a whole warp that calls together -- the
    // usual shape of a caller's kernel, one key per thread: the warp reads each key's home group as one
    // 128-byte request, 4 lanes taking 32 bytes each (the layout the bulk kernels read), instead of each
    // thread issuing eight 16-byte loads per group, which holds a table in DRAM to about a third of the
    // memory's random-read rate.  A key not decided in its home group (the group full of other keys), an
    // out-of-band key, and the lanes of a partial warp go on alone.
    __device__ int64_t
    find_slot_warp(key_type key, int64_t home, mapped_type* out) const
    {
        constexpr int S = 32 / C::slot_bytes; // slots per 32-byte sector
        constexpr bool is_map = detail::kind_traits<KIND>::is_map;
        int64_t slot = -1;
        bool read_value = true; // found alone: the value is read from the slot
        mapped_type val{};
        const bool probe = !is_special(key);
        if (__activemask() == 0xffffffffu)
        {
            unsigned lane;
            asm("mov.u32 %0, %%laneid;" : "=r"(lane));
            const int tbase = static_cast<int>(lane & ~3u);
            const int q = static_cast<int>(lane & 3u);
            const long long my_home = probe ? static_cast<long long>(home) : 0ll;
            long long hr[4];
            uint32_t w[4][8];
#pragma unroll
            for (int r = 0; r < 4; ++r)
            {
                hr[r] = __shfl_sync(0xffffffffu, my_home, tbase + r);
                const char* p = static_cast<const char*>(v.slots) + hr[r] * detail::kGroupBytes + 32 * q;
                asm volatile("ld.global.cg.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                             : "=r"(w[r][0]), "=r"(w[r][1]), "=r"(w[r][2]), "=r"(w[r][3]), "=r"(w[r][4]),
                               "=r"(w[r][5]), "=r"(w[r][6]), "=r"(w[r][7])
                             : "l"(p));
            }
            int64_t my_slot = -1;
            bool my_more = false;
#pragma unroll
            for (int r = 0; r < 4; ++r)
            {
                const key_type kr = __shfl_sync(0xffffffffu, key, tbase + r);
                unsigned mm = 0u, me = 0u;
#pragma unroll
                for (int s2 = 0; s2 < S; ++s2)
                {
                    const key_type k = sector_key(w[r], s2);
                    mm |= static_cast<unsigned>(k == kr) << s2;
                    me |= static_cast<unsigned>(k == C::empty_key) << s2;
                }
                const unsigned tm = (__ballot_sync(0xffffffffu, mm != 0u) >> tbase) & 0xFu;
                const unsigned te = (__ballot_sync(0xffffffffu, me != 0u) >> tbase) & 0xFu;
                const int owner = tm != 0u ? __ffs(tm) - 1 : 0;
                const unsigned om = __shfl_sync(0xffffffffu, mm, tbase + owner);
                mapped_type vr{};
                if constexpr (is_map)
                {
                    // the first matching slot's value, selected over constant indices (the sector stays in registers)
                    const int first = mm != 0u ? __ffs(mm) - 1 : 0;
                    mapped_type mine{};
#pragma unroll
                    for (int s2 = 0; s2 < S; ++s2)
                    {
                        if (s2 == first)
                        {
                            mine = sector_value(w[r], s2);
                        }
                    }
                    vr = __shfl_sync(0xffffffffu, mine, tbase + owner);
                }
                if (q == r)
                {
                    my_slot = tm != 0u ? hr[r] * G + owner * S + (__ffs(om) - 1) : -1;
                    my_more = tm == 0u && te == 0u;
                    val = vr;
                }
            }
            if (!probe)
            {
                slot = find_slot_home(key, home);
            }
            else if (my_more)
            {
                slot = find_slot_home(key, detail::next_group(home, v.num_groups));
            }
            else
            {
                slot = my_slot;
                read_value = false;
            }
        }
        else
        {
            slot = find_slot_home(key, home);
        }
        if constexpr (is_map)
        {
            if (out != nullptr && slot >= 0)
            {
                *out = read_value ? __ldcg(reinterpret_cast<const mapped_type*>(slot_ptr(slot) +
                                                                              detail::kind_traits<KIND>::val_offset))
                                  : val;
            }
        }
        return slot;
    }

    // find_slot along the probe sequence of home group `home` (the key's own).
    __device__ int64_t
    find_slot_home(key_type key, int64_t home) const
    {
        if (is_special(key))
        {
            const int s = key == C::empty_key ? 0 : 1;
            unsigned st = *reinterpret_cast<volatile unsigned*>(&header()->special_state[s]);
            return st == 1u ? special_slot(key) : -1;
        }
        int64_t g = home;
        for (int64_t probes = 0; probes < v.num_groups; ++probes)
        {
            const uint4* p = group_ptr(g);
            bool any_empty = false;
#pragma unroll
            for (int l = 0; l < detail::kTileLanes; ++l)
            {
                const uint4 d = __ldcg(p + l);
#pragma unroll
                for (int s = 0; s < SPL; ++s)
                {
                    const key_type k = detail::key_in_lane<KIND>(d, s);
                    if (k == key)
                    {
                        return g * G + l * SPL + s;
                    }
                    any_empty |= (k == C::empty_key);
                }
            }
            if (any_empty)
            {
                return -1;
            }
            g = detail::next_group(g, v.num_groups);
        }
        return -1;
    }

    // Slot of the stored key k for which eq(k) holds, searched along the probe sequence of the home group of
    // `hash` (heterogeneous lookup: a key-like value with the same hash as the key it equals), or -1.
    template <class Eq>
    __device__ int64_t
    find_slot_if(uint64_t hash, Eq eq) const
    {
        for (int s = 0; s < 2; ++s)
        {
            const key_type k = s == 0 ? C::empty_key : C::tomb_key;
            if (*reinterpret_cast<volatile unsigned*>(&header()->special_state[s]) == 1u && eq(k))
            {
                return special_slot(k);
            }
        }
        int64_t g = detail::group_of_bucket(detail::fibonacci_bucket(hash, v.bucket_bits), v.bucket_bits, v.num_groups);
        for (int64_t probes = 0; probes < v.num_groups; ++probes)
        {
            const uint4* p = group_ptr(g);
            bool any_empty = false;
#pragma unroll
            for (int l = 0; l < detail::kTileLanes; ++l)
            {
                const uint4 d = __ldcg(p + l);
#pragma unroll
                for (int s = 0; s < SPL; ++s)
                {
                    const key_type k = detail::key_in_lane<KIND>(d, s);
                    if (k == C::empty_key)
                    {
                        any_empty = true;
                    }
                    else if (k != C::tomb_key && eq(k))
                    {
                        return g * G + l * SPL + s;
                    }
                }
            }
            if (any_empty)
            {
                return -1;
            }
            g = detail::next_group(g, v.num_groups);
        }
        return -1;
    }

    __device__ __forceinline__ bool
    contains(key_type key) const
    {
        return find_slot(key) >= 0;
    }

    __device__ __forceinline__ int64_t
    count(key_type key) const
    {
        return contains(key) ? 1 : 0;
    }

    // find(key): true and *out = mapped value when present (maps); sets ignore out.
    __device__ bool
    find(key_type key, mapped_type* out) const
    {
        return find_slot_warp(key, home_group(key), out) >= 0;
    }

    __device__ void
    unlock_group(int64_t g, bool fence = true) const
    {
        if (fence)
        {
            detail::fence_acq_rel_gpu();
        }
        // held (bit 0 set) -> free with the next version: word + 1
        atomicAdd(v.insert_locks + (static_cast<uint64_t>(g) & static_cast<uint64_t>(v.lock_mask)), 1u);
    }

    // The stripe lock word of home group g: bit 0 held, bits 1-31 a version that every release advances.
    __device__ __forceinline__ unsigned int*
    lock_word(int64_t g) const
    {
        return v.insert_locks + (static_cast<uint64_t>(g) & static_cast<uint64_t>(v.lock_mask));
    }

    // The slot's current bytes as four words (unused words all ones).
    __device__ void
    read_slot(int64_t slot, uint32_t (&w)[4]) const
    {
        w[0] = w[1] = w[2] = w[3] = ~0u;
        if constexpr (C::slot_bytes == 16)
        {
            const uint4 d = __ldcg(reinterpret_cast<const uint4*>(slot_ptr(slot)));
            w[0] = d.x;
            w[1] = d.y;
            w[2] = d.z;
            w[3] = d.w;
        }
        else if constexpr (C::slot_bytes == 8)
        {
            const uint2 d = __ldcg(reinterpret_cast<const uint2*>(slot_ptr(slot)));
            w[0] = d.x;
            w[1] = d.y;
        }
        else
        {
            w[0] = __ldcg(reinterpret_cast<const unsigned int*>(slot_ptr(slot)));
        }
    }

    // The key along its probe sequence from group home, up to the first group holding a never-used slot:
    // true when present; else target = the first free slot on the way (erased below max_size(), or never
    // used; -1 when there is none) and whether it is an erased one.
    __device__ __forceinline__ bool
    scan_for_insert(key_type key, int64_t home, int64_t& target, bool& target_tomb) const
    {
        target = -1;
        target_tomb = false;
        return scan_for_insert_from(key, home, target, target_tomb);
    }

    // scan_for_insert from group g0 on, with target / target_tomb as found before g0 (target -1: none yet).
    __device__ bool
    scan_for_insert_from(key_type key, int64_t g0, int64_t& target, bool& target_tomb) const
    {
        int64_t g = g0;
        for (int64_t probes = 0; probes < v.num_groups; ++probes)
        {
            const uint4* p = group_ptr(g);
            bool any_empty = false;
            bool present = false;
#pragma unroll
            for (int l = 0; l < detail::kTileLanes; ++l)
            {
                const uint4 d = __ldcg(p + l);
#pragma unroll
                for (int s = 0; s < SPL; ++s)
                {
                    const key_type k = detail::key_in_lane<KIND>(d, s);
                    const int64_t slot = g * G + l * SPL + s;
                    present |= k == key;
                    any_empty |= k == C::empty_key;
                    if (target < 0 && (k == C::empty_key || (k == C::tomb_key && slot < v.total_count)))
                    {
                        target = slot;
                        target_tomb = k == C::tomb_key;
                    }
                }
            }
            if (present)
            {
                return true;
            }
            if (any_empty)
            {
                break;
            }
            g = detail::next_group(g, v.num_groups);
        }
        return false;
    }

    // scan_for_insert for the keys of a whole warp that calls together: the home groups are read as in
    // find_slot_warp (one 128-byte request per key); a key whose home group is full of other keys, and the
    // lanes of a partial warp, go on alone.
    __device__ bool
    scan_for_insert_warp(key_type key, int64_t home, int64_t& target, bool& target_tomb) const
    {
        constexpr int S = 32 / C::slot_bytes;
        if (__activemask() != 0xffffffffu)
        {
            return scan_for_insert(key, home, target, target_tomb);
        }
        unsigned lane;
        asm("mov.u32 %0, %%laneid;" : "=r"(lane));
        const int tbase = static_cast<int>(lane & ~3u);
        const int q = static_cast<int>(lane & 3u);
        long long hr[4];
        uint32_t w[4][8];
#pragma unroll
        for (int r = 0; r < 4; ++r)
        {
            hr[r] = __shfl_sync(0xffffffffu, static_cast<long long>(home), tbase + r);
            const char* p = static_cast<const char*>(v.slots) + hr[r] * detail::kGroupBytes + 32 * q;
            asm volatile("ld.global.cg.v8.u32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                         : "=r"(w[r][0]), "=r"(w[r][1]), "=r"(w[r][2]), "=r"(w[r][3]), "=r"(w[r][4]), "=r"(w[r][5]),
                           "=r"(w[r][6]), "=r"(w[r][7])
                         : "l"(p));
        }
        bool present = false, any_empty = false;
        target = -1;
        target_tomb = false;
#pragma unroll
        for (int r = 0; r < 4; ++r)
        {
            const key_type kr = __shfl_sync(0xffffffffu, key, tbase + r);
            const int64_t first_slot = hr[r] * G + q * S;
            unsigned mm = 0u, me = 0u, mt = 0u;
#pragma unroll
            for (int s2 = 0; s2 < S; ++s2)
            {
                const key_type k = sector_key(w[r], s2);
                mm |= static_cast<unsigned>(k == kr) << s2;
                me |= static_cast<unsigned>(k == C::empty_key) << s2;
                mt |= static_cast<unsigned>(k == C::tomb_key && first_slot + s2 < v.total_count) << s2;
            }
            const unsigned tm = (__ballot_sync(0xffffffffu, mm != 0u) >> tbase) & 0xFu;
            const unsigned te = (__ballot_sync(0xffffffffu, me != 0u) >> tbase) & 0xFu;
            const unsigned tf = (__ballot_sync(0xffffffffu, (me | mt) != 0u) >> tbase) & 0xFu;
            // the group's first free slot, erased or never used, in slot order
            const int fo = tf != 0u ? __ffs(tf) - 1 : 0;
            const unsigned ff = __shfl_sync(0xffffffffu, me | mt, tbase + fo);
            const unsigned ft = __shfl_sync(0xffffffffu, mt, tbase + fo);
            if (q == r)
            {
                present = tm != 0u;
                any_empty = te != 0u;
                if (tf != 0u)
                {
                    const int sl = __ffs(ff) - 1;
                    target = hr[r] * G + fo * S + sl;
                    target_tomb = ((ft >> sl) & 1u) != 0u;
                }
            }
        }
        if (present)
        {
            return true;
        }
        if (any_empty)
        {
            return false;
        }
        return scan_for_insert_from(key, detail::next_group(home, v.num_groups), target, target_tomb);
    }

    // The stripe lock of home group `home` for an insert (for_insert) or an erase of `key`: 1 when taken, 0
    // when the call was settled while waiting -- the key turned up present (insert) or absent (erase), checked
    // every 16 polls, so a crowd of calls on one key drains as soon as the first is done instead of passing
    // the lock on one by one --, -1 when the bounded wait gave up.  The lock word is read before each
    // compare-and-swap, so waiters load from L2 instead of all issuing atomics on one address.
    __device__ int
    lock_or_settled(int64_t home, key_type key, bool for_insert) const
    {
        unsigned int* l = lock_word(home);
        unsigned int backoff = 32;
        for (long long polls = 0; polls < detail::kWaitLimit; ++polls)
        {
            const unsigned int x = *reinterpret_cast<volatile unsigned int*>(l);
            if ((x & 1u) == 0u && atomicCAS(l, x, x | 1u) == x)
            {
                detail::fence_acq_rel_gpu();
                return 1;
            }
            if ((polls & 15) == 15 && (find_slot_home(key, home) >= 0) == for_insert)
            {
                return 0;
            }
            __nanosleep(backoff);
            backoff = backoff < 256 ? backoff * 2 : 256;
        }
        return -1;
    }

    // ---- the reference's excess-list accounting (v.bucket_heads != nullptr) ----
    // The reference stores a new key in its bucket's own slot when that slot is free, else in a slot taken
    // from its excess list; its insert loop refuses every insert once the table is full or that list is
    // empty (unordered_base_detail.cuh:708-809, 958-994), and an erase frees the bucket's slot or gives the
    // excess slot back (:811-913).  The view keeps the same state: bucket_heads (a bit per bucket: a key holds
    // the bucket's own slot), slot_heads (a bit per slot: the key stored there is that key) and the header's
    // excess_used.  Every change for a key of bucket b happens under the stripe lock of b's home group, which
    // all keys of b share.
    __device__ __forceinline__ bool
    accounting() const
    {
        return v.bucket_heads != nullptr;
    }

    // the reference's loop guard (:980-981): full(), or no excess slot left
    __device__ __forceinline__ bool
    refuses_all() const
    {
        return *reinterpret_cast<volatile unsigned long long*>(&header()->excess_used) >=
                       static_cast<unsigned long long>(v.excess_count) ||
               *reinterpret_cast<volatile unsigned long long*>(&header()->size) >=
                       static_cast<unsigned long long>(v.total_count);
    }

    // For a new key of bucket b: 1 = it takes the bucket's own slot, 0 = an excess slot, -1 = refused.  With
    // may_take_bucket false the key takes an excess slot even when the bucket's own is free (a bulk call in
    // which an earlier new key of the same bucket takes that slot).
    __device__ int
    take_bucket_or_excess(int64_t b, bool may_take_bucket = true) const
    {
        if (refuses_all())
        {
            return -1;
        }
        const unsigned bit = 1u << (b & 31);
        if (may_take_bucket && (atomicOr(v.bucket_heads + (b >> 5), bit) & bit) == 0u)
        {
            return 1;
        }
        if (defer != nullptr)
        {
            defer->excess += 1; // a bulk call that cannot reach the end of the list: counted at its end
            return 0;
        }
        if (atomicAdd(&header()->excess_used, 1ull) < static_cast<unsigned long long>(v.excess_count))
        {
            return 0;
        }
        atomicAdd(&header()->excess_used, ~0ull);
        return -1;
    }

    // Undoes take_bucket_or_excess(b) == held for an insert that stored nothing.
    __device__ void
    give_back(int64_t b, int held) const
    {
        if (held == 1)
        {
            atomicAnd(v.bucket_heads + (b >> 5), ~(1u << (b & 31)));
        }
        else if (held == 0)
        {
            add_excess(-1);
        }
    }

    __device__ __forceinline__ void
    mark_bucket_slot(int64_t slot) const
    {
        atomicOr(v.slot_heads + (slot >> 5), 1u << (slot & 31));
    }

    // Before the key of bucket b at `slot` is erased: clears the slot's bit and returns whether it was set.
    __device__ __forceinline__ bool
    unmark_bucket_slot(int64_t slot) const
    {
        const unsigned bit = 1u << (slot & 31);
        return (atomicAnd(v.slot_heads + (slot >> 5), ~bit) & bit) != 0u;
    }

    // After that key is erased: the bucket's own slot becomes free, or its excess slot goes back.
    __device__ void
    release(int64_t b, bool was_bucket_slot) const
    {
        if (was_bucket_slot)
        {
            atomicAnd(v.bucket_heads + (b >> 5), ~(1u << (b & 31)));
        }
        else
        {
            add_excess(-1);
        }
    }

    // Insert under the home group's stripe lock: erased slots are reused.  Returns the slot, or -1 (present,
    // refused -- no free slot in the table --, or the lock wait gave up, which sets an error bit).  As the
    // reference checks contains() and full() before it locks (unordered_base_detail.cuh:708-720, :958-994),
    // a key found present, or a table with no free slot along the key's probe sequence, is decided by one
    // scan without the lock, so inserts of present keys and inserts into a full table do not queue on it.
    __device__ int64_t
    insert_slot_locked(key_type key, mapped_type mapped, int64_t b, bool may_take_bucket = true) const
    {
        const int64_t home = detail::group_of_bucket(static_cast<uint64_t>(b), v.bucket_bits, v.num_groups);
        // the lock's version before the lock-free scan: taking the lock at that same version means no insert
        // of this stripe -- no insert of this key -- completed since, so the scan's answer still holds (erases
        // take no lock, but they only turn keys into erased slots)
        unsigned int* l = lock_word(home);
        unsigned int v0;
        // an acquire load: the scan's reads come after it, so a release seen here is seen by the scan too
        asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v0) : "l"(l) : "memory");
        int64_t pre_target = -1;
        bool pre_tomb = false;
        if (scan_for_insert_warp(key, home, pre_target, pre_tomb))
        {
            return -1; // present
        }
        if (pre_target < 0 || (accounting() && refuses_all()))
        {
            add_refused();
            return -1;
        }
        bool scanned = false; // the prescan's target is current
        int locked;
        if ((v0 & 1u) == 0u && atomicCAS(l, v0, v0 | 1u) == v0)
        {
            // no fence: nothing is read under the lock on this path, and the claim below waits for this
            // compare-and-swap's answer
            locked = 1;
            scanned = true;
        }
        else
        {
            locked = lock_or_settled(home, key, true);
        }
        if (locked == 0)
        {
            return -1; // present: inserted by another thread while this one waited
        }
        if (locked < 0)
        {
            atomicOr(&header()->error, detail::kErrRetry);
            return -1;
        }
        int64_t result = -1;
        bool refused = false;
        int held = -1; // accounting: what take_bucket_or_excess gave this key
        for (int attempt = 0; attempt < 65536; ++attempt)
        {
            int64_t target = pre_target;
            bool target_tomb = pre_tomb;
            if (!scanned)
            {
                if (scan_for_insert(key, home, target, target_tomb))
                {
                    break; // present
                }
            }
            scanned = false; // a lost claim below reads the chain again
            if (target < 0)
            {
                refused = true;
                break;
            }
            if (accounting() && held < 0)
            {
                held = take_bucket_or_excess(b, may_take_bucket);
                if (held < 0)
                {
                    refused = true;
                    break;
                }
            }
            uint32_t image[4];
            if (target_tomb)
            {
                read_slot(target, image);
                if (detail::key_in_lane<KIND>(make_uint4(image[0], image[1], image[2], image[3]), 0) != C::tomb_key)
                {
                    continue; // taken since the scan: scan again
                }
            }
            else
            {
                image[0] = image[1] = image[2] = image[3] = ~0u;
            }
            key_type old;
            if (detail::claim_slot_image<KIND>(slot_ptr(target), image, key, mapped, old))
            {
                add_size(1);
                if (target_tomb)
                {
                    add_tombs(-1);
                }
                if (held == 1)
                {
                    mark_bucket_slot(target);
                }
                result = target;
                break;
            }
            if (old == key)
            {
                break;
            }
            // another key took the slot: scan again
        }
        if (result < 0 && held >= 0)
        {
            give_back(b, held);
        }
        // the claim's compare-and-swap has answered, so the next holder sees the key; the accounting's bit
        // updates are not waited for, and need the fence
        unlock_group(home, accounting());
        if (refused)
        {
            add_refused();
        }
        return result;
    }

    // insert(value) / emplace(key, mapped): the slot this call stored the key in, or -1 when the key
    // was already present or no free slot was left (the reference returns (end(), false)).
    __device__ __forceinline__ int64_t
    insert_slot(key_type key, mapped_type mapped = mapped_type{}) const
    {
        return insert_slot_bucket(key, mapped, bucket(key));
    }

    // insert_slot for a key whose hash the caller computed (the reference's Hash applied by the caller).
    __device__ __forceinline__ int64_t
    insert_slot_hashed(key_type key, uint64_t hash, mapped_type mapped = mapped_type{}) const
    {
        return insert_slot_bucket(key, mapped, static_cast<int64_t>(detail::fibonacci_bucket(hash, v.bucket_bits)));
    }

    // An out-of-band key (stored outside the probe groups) under the accounting: the stripe lock of its home
    // group orders it with the other keys of its bucket.
    __device__ int64_t
    insert_special_counted(key_type key, mapped_type mapped, int64_t b, bool may_take_bucket) const
    {
        const int s = key == C::empty_key ? 0 : 1;
        if (*reinterpret_cast<volatile unsigned*>(&header()->special_state[s]) == 1u)
        {
            return -1;
        }
        if (refuses_all())
        {
            add_refused();
            return -1;
        }
        const int64_t home = detail::group_of_bucket(static_cast<uint64_t>(b), v.bucket_bits, v.num_groups);
        const int locked = lock_or_settled(home, key, true);
        if (locked <= 0)
        {
            if (locked < 0)
            {
                atomicOr(&header()->error, detail::kErrRetry);
            }
            return -1;
        }
        int64_t result = -1;
        const int held = take_bucket_or_excess(b, may_take_bucket);
        if (held < 0)
        {
            add_refused();
        }
        else if (atomicCAS(&header()->special_state[s], 0u, 2u) == 0u)
        {
            store_slot(special_slot(key), key, mapped);
            __threadfence();
            atomicExch(&header()->special_state[s], 1u);
            add_size(1);
            if (held == 1)
            {
                mark_bucket_slot(special_slot(key));
            }
            result = special_slot(key);
        }
        else
        {
            give_back(b, held);
        }
        unlock_group(home);
        return result;
    }

    // Insert of a bulk call with the accounting on that cannot reach the refusal (the caller checked that the
    // size and the keys in excess slots stay below their limits whatever the call does) and runs no erase:
    // no lock, as in the bulk kernels -- only free slots disappear during the launch, and each insert reads
    // every slot before the one it claims, so a key is stored once.  The stored copy then takes its bucket's
    // own slot when it is the bucket's first new key (first_new) and the slot is free, else an excess slot.
    __device__ int64_t
    insert_slot_quiet(key_type key, mapped_type mapped, int64_t b, bool first_new) const
    {
        int64_t slot = -1;
        if (is_special(key))
        {
            const int s = key == C::empty_key ? 0 : 1;
            if (atomicCAS(&header()->special_state[s], 0u, 2u) != 0u)
            {
                return -1;
            }
            store_slot(special_slot(key), key, mapped);
            __threadfence();
            atomicExch(&header()->special_state[s], 1u);
            slot = special_slot(key);
        }
        else
        {
            const int64_t home = detail::group_of_bucket(static_cast<uint64_t>(b), v.bucket_bits, v.num_groups);
            for (int attempt = 0; attempt < 65536 && slot < 0; ++attempt)
            {
                int64_t target = -1;
                bool target_tomb = false;
                // the first read with the warp (all lanes arrive here together in a bulk kernel's step)
                if (attempt == 0 ? scan_for_insert_warp(key, home, target, target_tomb)
                                 : scan_for_insert(key, home, target, target_tomb))
                {
                    return -1; // present
                }
                if (target < 0)
                {
                    add_refused();
                    return -1;
                }
                uint32_t image[4];
                if (target_tomb)
                {
                    read_slot(target, image);
                    if (detail::key_in_lane<KIND>(make_uint4(image[0], image[1], image[2], image[3]), 0) != C::tomb_key)
                    {
                        continue; // taken since the scan
                    }
                }
                else
                {
                    image[0] = image[1] = image[2] = image[3] = ~0u;
                }
                key_type old;
                if (detail::claim_slot_image<KIND>(slot_ptr(target), image, key, mapped, old))
                {
                    if (target_tomb)
                    {
                        add_tombs(-1);
                    }
                    slot = target;
                }
                else if (old == key)
                {
                    return -1;
                }
            }
            if (slot < 0)
            {
                atomicOr(&header()->error, detail::kErrRetry);
                return -1;
            }
        }
        add_size(1);
        const unsigned bit = 1u << (b & 31);
        if (first_new && (atomicOr(v.bucket_heads + (b >> 5), bit) & bit) == 0u)
        {
            mark_bucket_slot(slot);
        }
        else
        {
            add_excess(1);
        }
        return slot;
    }

    // insert_slot for a key of bucket b; may_take_bucket as in take_bucket_or_excess (accounting only).
    __device__ int64_t
    insert_slot_bucket(key_type key, mapped_type mapped, int64_t b, bool may_take_bucket = true) const
    {
        if (is_special(key) && accounting())
        {
            return insert_special_counted(key, mapped, b, may_take_bucket);
        }
        if (is_special(key))
        {
            const int s = key == C::empty_key ? 0 : 1;
            if (atomicCAS(&header()->special_state[s], 0u, 2u) != 0u)
            {
                return -1;
            }
            store_slot(special_slot(key), key, mapped);
            __threadfence();
            atomicExch(&header()->special_state[s], 1u);
            add_size(1);
            return special_slot(key);
        }
        if (v.insert_locks != nullptr)
        {
            return insert_slot_locked(key, mapped, b, may_take_bucket);
        }
        int64_t g = detail::group_of_bucket(static_cast<uint64_t>(b), v.bucket_bits, v.num_groups);
        int64_t steps = 0;
        const int64_t limit = v.num_groups + 4096;
        while (steps++ < limit)
        {
            const uint4* p = group_ptr(g);
            int64_t target = -1;
#pragma unroll
            for (int l = 0; l < detail::kTileLanes; ++l)
            {
                const uint4 d = __ldcg(p + l);
#pragma unroll
                for (int s = 0; s < SPL; ++s)
                {
                    const key_type k = detail::key_in_lane<KIND>(d, s);
                    if (k == key)
                    {
                        return -1;
                    }
                    if (target < 0 && k == C::empty_key)
                    {
                        target = g * G + l * SPL + s;
                    }
                }
            }
            if (target < 0)
            {
                g = detail::next_group(g, v.num_groups);
                if (steps > v.num_groups)
                {
                    break;
                }
                continue;
            }
            key_type old;
            const uint32_t never_used[4] = { ~0u, ~0u, ~0u, ~0u };
            if (detail::claim_slot_image<KIND>(slot_ptr(target), never_used, key, mapped, old))
            {
                add_size(1);
                return target;
            }
            if (old == key)
            {
                return -1;
            }
            // lost the slot to another key: rescan the same group
        }
        add_refused();
        return -1;
    }

    __device__ __forceinline__ bool
    insert(key_type key, mapped_type mapped = mapped_type{}) const
    {
        return insert_slot(key, mapped) >= 0;
    }

    // bucket_size(n): stored keys whose reference bucket is n (unordered_base_detail.cuh:566-593).  They
    // all sit on the probe sequence of n's home group before its first group holding a never-used slot.
    __device__ int64_t
    bucket_size(int64_t n) const
    {
        if (n < 0 || n >= (int64_t{ 1 } << v.bucket_bits))
        {
            return 0; // no such bucket (the reference requires n < bucket_count())
        }
        int64_t g = detail::group_of_bucket(static_cast<uint64_t>(n), v.bucket_bits, v.num_groups);
        int64_t c = 0;
        for (int64_t probes = 0; probes < v.num_groups; ++probes)
        {
            const uint4* p = group_ptr(g);
            bool any_empty = false;
#pragma unroll
            for (int l = 0; l < detail::kTileLanes; ++l)
            {
                const uint4 d = __ldcg(p + l);
#pragma unroll
                for (int s = 0; s < SPL; ++s)
                {
                    const key_type k = detail::key_in_lane<KIND>(d, s);
                    if (k == C::empty_key)
                    {
                        any_empty = true;
                    }
                    else if (k != C::tomb_key && g * G + l * SPL + s < v.total_count && bucket(k) == n)
                    {
                        ++c;
                    }
                }
            }
            if (any_empty)
            {
                break;
            }
            g = detail::next_group(g, v.num_groups);
        }
        for (int s = 0; s < 2; ++s)
        {
            const key_type k = s == 0 ? C::empty_key : C::tomb_key;
            if (*reinterpret_cast<volatile unsigned*>(&header()->special_state[s]) == 1u && bucket(k) == n)
            {
                ++c;
            }
        }
        return c;
    }

    __device__ __forceinline__ bool
    emplace(key_type key, mapped_type mapped = mapped_type{}) const
    {
        return insert(key, mapped);
    }

    // erase(key): 1 when this call removed the key, else 0.
    __device__ __forceinline__ int64_t
    erase(key_type key) const
    {
        return erase_bucket(key, bucket(key));
    }

    // erase for a key whose hash the caller computed.
    __device__ __forceinline__ int64_t
    erase_hashed(key_type key, uint64_t hash) const
    {
        return erase_bucket(key, static_cast<int64_t>(detail::fibonacci_bucket(hash, v.bucket_bits)));
    }

    // Erase of a bulk erase call with the accounting on: no insert runs in the launch, so no lock -- the slot's
    // bit is read after the swap that erased the key, which only one erase of a key wins.
    __device__ int64_t
    erase_quiet(key_type key, int64_t b) const
    {
        const int64_t slot = find_slot_warp(
                key, detail::group_of_bucket(static_cast<uint64_t>(b), v.bucket_bits, v.num_groups), nullptr);
        if (slot < 0)
        {
            return 0;
        }
        if (is_special(key))
        {
            if (atomicCAS(&header()->special_state[key == C::empty_key ? 0 : 1], 1u, 0u) != 1u)
            {
                return 0;
            }
        }
        else if (cas_key(slot, key, C::tomb_key) == key)
        {
            add_tombs(1);
        }
        else
        {
            return 0;
        }
        add_size(-1);
        release(b, unmark_bucket_slot(slot));
        return 1;
    }

    __device__ __forceinline__ int64_t
    erase_quiet_hashed(key_type key, uint64_t hash) const
    {
        return erase_quiet(key, static_cast<int64_t>(detail::fibonacci_bucket(hash, v.bucket_bits)));
    }

    // erase under the accounting: the stripe lock of the key's home group, then the slot's bits.
    __device__ int64_t
    erase_counted(key_type key, int64_t b) const
    {
        const int64_t home = detail::group_of_bucket(static_cast<uint64_t>(b), v.bucket_bits, v.num_groups);
        if (find_slot_warp(key, home, nullptr) < 0)
        {
            return 0;
        }
        const int locked = lock_or_settled(home, key, false);
        if (locked <= 0)
        {
            if (locked < 0)
            {
                atomicOr(&header()->error, detail::kErrRetry);
            }
            return 0;
        }
        int64_t r = 0;
        const int64_t slot = find_slot_home(key, home);
        if (slot >= 0)
        {
            // the bit goes before the slot can be reused by another bucket's key
            const bool was_bucket_slot = unmark_bucket_slot(slot);
            bool erased = false;
            if (is_special(key))
            {
                erased = atomicCAS(&header()->special_state[key == C::empty_key ? 0 : 1], 1u, 0u) == 1u;
            }
            else if (cas_key(slot, key, C::tomb_key) == key)
            {
                add_tombs(1);
                erased = true;
            }
            if (erased)
            {
                add_size(-1);
                release(b, was_bucket_slot);
                r = 1;
            }
            else if (was_bucket_slot)
            {
                mark_bucket_slot(slot);
            }
        }
        unlock_group(home);
        return r;
    }

    __device__ int64_t
    erase_bucket(key_type key, int64_t b) const
    {
        if (accounting())
        {
            return erase_counted(key, b);
        }
        if (is_special(key))
        {
            const int s = key == C::empty_key ? 0 : 1;
            if (atomicCAS(&header()->special_state[s], 1u, 0u) == 1u)
            {
                add_size(-1);
                return 1;
            }
            return 0;
        }
        const int64_t slot = find_slot_warp(
                key, detail::group_of_bucket(static_cast<uint64_t>(b), v.bucket_bits, v.num_groups), nullptr);
        if (slot < 0)
        {
            return 0;
        }
        if (cas_key(slot, key, C::tomb_key) == key)
        {
            add_size(-1);
            add_tombs(1);
            return 1;
        }
        return 0;
    }

    __device__ __forceinline__ key_type
    cas_key(int64_t slot, key_type expected, key_type desired) const
    {
        if constexpr (sizeof(key_type) == 8)
        {
            return static_cast<key_type>(atomicCAS(reinterpret_cast<unsigned long long*>(slot_ptr(slot)),
                                                   static_cast<unsigned long long>(expected),
                                                   static_cast<unsigned long long>(desired)));
        }
        else
        {
            return static_cast<key_type>(atomicCAS(reinterpret_cast<unsigned int*>(slot_ptr(slot)),
                                                   static_cast<unsigned int>(expected),
                                                   static_cast<unsigned int>(desired)));
        }
    }

    __device__ __forceinline__ void
    store_slot(int64_t slot, key_type key, mapped_type mapped) const
    {
        *reinterpret_cast<volatile key_type*>(slot_ptr(slot)) = key;
        if constexpr (detail::kind_traits<KIND>::is_map)
        {
            *reinterpret_cast<volatile mapped_type*>(slot_ptr(slot) + detail::kind_traits<KIND>::val_offset) = mapped;
        }
    }
};

using unordered_set_u32_ref = unordered_ref<SG_SET_U32>;
using unordered_set_u64_ref = unordered_ref<SG_SET_U64>;
using unordered_map_u64_u32_ref = unordered_ref<SG_MAP_U64_U32>;
using unordered_map_u64_u64_ref = unordered_ref<SG_MAP_U64_U64>;
using unordered_map_u32_u32_ref = unordered_ref<SG_MAP_U32_U32>;
using unordered_map_u32_u64_ref = unordered_ref<SG_MAP_U32_U64>;

} // namespace sg

#endif

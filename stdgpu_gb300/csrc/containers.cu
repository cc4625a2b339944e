// vector<T>::push_back, deque<T>::push_back / pop_front and bitset::count for GB300.
//
// vector / deque replace the reference's per-element global atomic plus slot
// spin lock (src/stdgpu/impl/vector_detail.cuh:181-238,
// src/stdgpu/impl/deque_detail.cuh:202-258, 388-446) with one reservation per
// tile of 2048 elements: the warps ballot, one warp scans the counts, one
// thread adds the tile's total to the shared counter and every element takes
// its rank.  A counter that every warp hits once saturates near 0.5 G updates
// a second on one address; once per tile it is no longer the bound.
//
// The deque is a ring of tickets: push k and pop k use slot k mod capacity; a
// per-slot turn counter (the k-th push stores k+1 after writing the element,
// the k-th pop stores k+capacity after reading it) orders a pop after the push
// of the same ticket and a push after the pop one lap earlier.  Those waits are
// bounded: a wait that runs out sets an error bit and the operation reports
// failure instead of spinning on.
//
// bitset::count (src/stdgpu/impl/bitset_detail.cuh:388-404, count_block_bits
// :130-160) is a two-pass reduction: 16-byte loads and popc per thread, one
// partial per block, then one block sums the partials.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <new>

#include "sg_internal.cuh"
#include "stdgpu_gb300.h"
#include "stdgpu_gb300/detail/layout.cuh"

namespace sg
{
namespace detail
{

constexpr int kCThreads = 256;
SG_D unsigned
lanemask_lt()
{
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

template <typename T>
SG_D T
ld_stream(const T* p)
{
    return __ldcs(p);
}

// A ring slot's turn word read without ordering (a fence_gpu after the reads orders what follows), and
// stored without ordering (a fence_gpu before the stores orders what precedes).
SG_D unsigned
load_turn_relaxed(const unsigned* p)
{
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

SG_D void
store_turn_relaxed(unsigned* p, unsigned v)
{
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

SG_D void
fence_gpu()
{
    asm volatile("fence.acq_rel.gpu;" ::: "memory");
}

// ---------------------------------------------------------------- block reservations
//
// A block takes a tile of kItems x kCThreads elements, element tile + j * kCThreads + threadIdx.x being
// item j of the thread.  Each warp ballots its items and writes one count per (item, warp) into shared
// memory in element order; one warp scans the kItems * kWarps counts, so every element learns its rank
// among the tile's selected elements and the tile makes one reservation on the shared counter.

constexpr int kItems = 8;
constexpr int kWarps = kCThreads / 32;
constexpr int kCounts = kItems * kWarps; // 64: two per lane of the scanning warp
constexpr int64_t kTileElems = int64_t{ kItems } * kCThreads;
static_assert(kCounts == 64, "the scan gives each lane two counts");

// Exclusive scan of cnt[0, 64) in place by one warp; returns the total to every lane.
SG_D unsigned
scan_counts(unsigned* cnt, int lane)
{
    const unsigned a = cnt[2 * lane];
    const unsigned b = cnt[2 * lane + 1];
    unsigned s = a + b;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
        const unsigned t = __shfl_up_sync(0xffffffffu, s, d);
        if (lane >= d)
        {
            s += t;
        }
    }
    const unsigned excl = s - a - b;
    cnt[2 * lane] = excl;
    cnt[2 * lane + 1] = excl + a;
    return __shfl_sync(0xffffffffu, s, 31);
}

// ---------------------------------------------------------------- vector

// Bulk push_back tiles: kVecItems elements per thread, one reservation on the shared size counter per tile.
// Measured for 2^28 threads (30 % push): 4 items (1024-element tiles) 0.69 ms, 8 items 0.80 ms, 12 items
// 1.31 ms, 16 items 1.33 ms -- larger tiles cost registers and resident warps more than their fewer
// reservations save; 8 items with the values loaded after the reservation took 1.18 ms.
#ifndef SG_VEC_ITEMS
#define SG_VEC_ITEMS 4
#endif
constexpr int kVecItems = SG_VEC_ITEMS;
constexpr int kVecCounts = kVecItems * kWarps;
constexpr int64_t kVecTileElems = int64_t{ kVecItems } * kCThreads;
static_assert(kVecCounts % 32 == 0 && kVecCounts <= 32 * 8, "whole counts per lane of the scanning warp");

// Exclusive scan of cnt[0, kVecCounts) in place by one warp (kVecCounts / 32 consecutive counts per lane);
// returns the total to every lane.
SG_D unsigned
scan_vec_counts(unsigned* cnt, int lane)
{
    constexpr int per = kVecCounts / 32;
    unsigned v[per];
    unsigned sum = 0u;
#pragma unroll
    for (int k = 0; k < per; ++k)
    {
        v[k] = cnt[per * lane + k];
        sum += v[k];
    }
    unsigned incl = sum;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1)
    {
        const unsigned t = __shfl_up_sync(0xffffffffu, incl, d);
        if (lane >= d)
        {
            incl += t;
        }
    }
    unsigned run = incl - sum;
#pragma unroll
    for (int k = 0; k < per; ++k)
    {
        cnt[per * lane + k] = run;
        run += v[k];
    }
    return __shfl_sync(0xffffffffu, incl, 31);
}

// Bulk push_back: element i pushes values[i] where pred[i] != 0 (every element without pred).  Per tile the
// selected values are loaded before the tile's reservation, so their loads are in flight while warp 0 scans
// the counts and adds the tile's total to the size; a reservation past capacity fails the tile's elements
// there, as the reference's push_back fails past capacity() (its size is clamped when read,
// vector_detail.cuh:484-511).  Two count buffers alternate between tiles, so a tile needs two barriers.
template <typename T>
__global__ void __launch_bounds__(kCThreads)
k_vector_push_back(T* data, long long* size, int64_t cap, const T* values, const uint8_t* pred, int64_t n,
                   uint8_t* out_pushed)
{
    __shared__ unsigned cnt[2][kVecCounts];
    __shared__ long long s_base[2];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    int buf = 0;
    for (int64_t tile = static_cast<int64_t>(blockIdx.x) * kVecTileElems; tile < n;
         tile += static_cast<int64_t>(gridDim.x) * kVecTileElems, buf ^= 1)
    {
        unsigned masks[kVecItems];
        T vals[kVecItems];
#pragma unroll
        for (int j = 0; j < kVecItems; ++j)
        {
            const int64_t i = tile + j * kCThreads + threadIdx.x;
            const bool want = i < n && (pred == nullptr || pred[i] != 0);
            masks[j] = __ballot_sync(0xffffffffu, want);
            if (lane == 0)
            {
                cnt[buf][j * kWarps + warp] = __popc(masks[j]);
            }
            vals[j] = want ? ld_stream(values + i) : T{};
        }
        __syncthreads();
        if (warp == 0)
        {
            const unsigned total = scan_vec_counts(cnt[buf], lane);
            if (lane == 0)
            {
                // one reservation for the tile (vector_detail.cuh:186-195)
                s_base[buf] = total > 0 ? static_cast<long long>(atomicAdd(reinterpret_cast<unsigned long long*>(size),
                                                                           static_cast<unsigned long long>(total)))
                                        : -1;
            }
        }
        __syncthreads();
        const long long base = s_base[buf];
#pragma unroll
        for (int j = 0; j < kVecItems; ++j)
        {
            const int64_t i = tile + j * kCThreads + threadIdx.x;
            const bool want = (masks[j] >> lane) & 1u;
            const long long pos = base + cnt[buf][j * kWarps + warp] + __popc(masks[j] & lanemask_lt());
            const bool ok = want && base >= 0 && pos < cap;
            if (ok)
            {
                data[pos] = vals[j];
            }
            if (i < n && out_pushed != nullptr)
            {
                out_pushed[i] = static_cast<uint8_t>(ok);
            }
        }
        // no barrier: the next tile fills the other count buffer, and the one after passes two barriers
        // that every warp reaches only after reading this tile's counts
    }
}

// ---------------------------------------------------------------- deque

SG_D long long
atomic_add_ll(long long* p, long long v)
{
    return static_cast<long long>(
            atomicAdd(reinterpret_cast<unsigned long long*>(p), static_cast<unsigned long long>(v)));
}

// Reserves up to `want` units of `counter` below `bound` (grow) or above zero (!grow): a preemptive read,
// one add, and an undo of what did not fit (deque_detail.cuh:207-217 push_back, :393-404 pop_front).
SG_D long long
reserve(long long* counter, long long bound, long long want, bool grow)
{
    const long long cur = *reinterpret_cast<volatile long long*>(counter);
    if (grow ? cur >= bound : cur <= 0)
    {
        return 0;
    }
    const long long old = atomic_add_ll(counter, grow ? want : -want);
    const long long room = grow ? bound - old : old;
    const long long take = room <= 0 ? 0 : (room < want ? room : want);
    if (take < want)
    {
        atomic_add_ll(counter, grow ? take - want : want - take);
    }
    return take;
}

// Mixed launch: element i pushes values[i] when is_push[i] != 0 (or is_push == NULL), else pops.  Each
// tile reserves its pushes and its pops once; the tile's pushes take consecutive tickets in element
// order, and so do its pops.
// resident blocks per SM the mixed deque launch is compiled for (its fast path keeps 8 tickets per thread in
// registers); measured for 2^26 mixed ops: 4 blocks 1.60 ms, 5 blocks 1.40 ms, 6 blocks 1.27 ms, and the
// one-by-one protocol alone (every element's turn waited for and released in turn) 1.60 ms
#ifndef SG_DEQUE_MIN_BLOCKS
#define SG_DEQUE_MIN_BLOCKS 6
#endif
// 0: every element takes the one-by-one path (for comparison)
#ifndef SG_DEQUE_FAST
#define SG_DEQUE_FAST 1
#endif

template <typename T>
__global__ void __launch_bounds__(kCThreads, SG_DEQUE_MIN_BLOCKS)
k_deque_ops(T* data, unsigned* seq, deque_counters* c, int64_t cap, const uint8_t* is_push, const T* values,
            int64_t n, T* out_popped, uint8_t* out_ok)
{
    __shared__ unsigned cpush[kCounts];
    __shared__ unsigned cpop[kCounts];
    __shared__ unsigned mpush[kCounts]; // the ballots, so the wait loop below indexes no local array
    __shared__ unsigned mpop[kCounts];
    __shared__ long long s_push_ok, s_pop_ok;
    __shared__ unsigned long long s_push_t0, s_pop_t0;
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    for (int64_t tile = static_cast<int64_t>(blockIdx.x) * kTileElems; tile < n;
         tile += static_cast<int64_t>(gridDim.x) * kTileElems)
    {
#pragma unroll
        for (int j = 0; j < kItems; ++j)
        {
            const int64_t i = tile + j * kCThreads + threadIdx.x;
            const bool in = i < n;
            const bool push = in && (is_push == nullptr || is_push[i] != 0);
            const unsigned pm = __ballot_sync(0xffffffffu, push);
            const unsigned qm = __ballot_sync(0xffffffffu, in && !push);
            if (lane == 0)
            {
                cpush[j * kWarps + warp] = __popc(pm);
                cpop[j * kWarps + warp] = __popc(qm);
                mpush[j * kWarps + warp] = pm;
                mpop[j * kWarps + warp] = qm;
            }
        }
        __syncthreads();
        if (warp < 2)
        {
            const bool grow = warp == 0;
            const unsigned total = scan_counts(grow ? cpush : cpop, lane);
            if (lane == 0)
            {
                const long long ok = total > 0 ? reserve(grow ? &c->size : &c->avail, cap, total, grow) : 0;
                unsigned long long t0 = 0;
                if (ok > 0)
                {
                    t0 = atomicAdd(grow ? &c->end : &c->begin, static_cast<unsigned long long>(ok));
                    atomic_add_ll(grow ? &c->avail : &c->size, grow ? ok : -ok);
                }
                if (grow)
                {
                    s_push_ok = ok;
                    s_push_t0 = t0;
                }
                else
                {
                    s_pop_ok = ok;
                    s_pop_t0 = t0;
                }
            }
        }
        __syncthreads();
        const long long push_ok = s_push_ok;
        const long long pop_ok = s_pop_ok;
        const unsigned long long push_t0 = s_push_t0;
        const unsigned long long pop_t0 = s_pop_t0;
        // The thread's tickets: slot and low 32 bits of the ticket (a push waits for turn tk and leaves
        // tk + 1, a pop waits for tk + 1 and leaves tk + capacity; capacity < 2^31).  All turns are read at
        // once (relaxed, then one fence); when every one of them is already there -- the usual case, each
        // slot's previous operation having finished in an earlier tile or launch -- the elements are moved,
        // one fence orders those moves before the turns, and the turns are stored.  Otherwise the thread
        // takes its elements one by one with bounded waits, each releasing its turn at once, since one of
        // its elements may wait for a turn another of them leaves.
        unsigned pos[kItems];
        unsigned tk32[kItems];
        unsigned pushes = 0u; // bit j: item j is a push with a ticket
        unsigned pops = 0u;   // bit j: item j is a pop with a ticket
        bool ready = true;
#pragma unroll
        for (int j = 0; j < kItems; ++j)
        {
            const unsigned bit = 1u << lane;
            const unsigned pm = mpush[j * kWarps + warp];
            const unsigned qm = mpop[j * kWarps + warp];
            pos[j] = 0u;
            tk32[j] = 0u;
            unsigned want = 0u;
            bool live = false;
            if (pm & bit)
            {
                const long long r = cpush[j * kWarps + warp] + __popc(pm & lanemask_lt());
                if (r < push_ok)
                {
                    const unsigned long long tk = push_t0 + static_cast<unsigned long long>(r);
                    pos[j] = static_cast<unsigned>(tk % static_cast<unsigned long long>(cap));
                    tk32[j] = static_cast<unsigned>(tk);
                    want = tk32[j];
                    pushes |= 1u << j;
                    live = true;
                }
            }
            else if (qm & bit)
            {
                const long long r = cpop[j * kWarps + warp] + __popc(qm & lanemask_lt());
                if (r < pop_ok)
                {
                    const unsigned long long tk = pop_t0 + static_cast<unsigned long long>(r);
                    pos[j] = static_cast<unsigned>(tk % static_cast<unsigned long long>(cap));
                    tk32[j] = static_cast<unsigned>(tk);
                    want = tk32[j] + 1u;
                    pops |= 1u << j;
                    live = true;
                }
            }
            if (live)
            {
                const unsigned cur = load_turn_relaxed(seq + pos[j]); // independent loads, all in flight
                ready = ready & (cur == want) & (SG_DEQUE_FAST != 0);
            }
        }
        if (ready)
        {
            fence_gpu(); // the turns read above come before the element accesses below
#pragma unroll
            for (int j = 0; j < kItems; ++j)
            {
                const int64_t i = tile + j * kCThreads + threadIdx.x;
                if (pushes & (1u << j))
                {
                    data[pos[j]] = ld_stream(values + i);
                }
                else if (pops & (1u << j))
                {
                    const T v = __ldcg(data + pos[j]);
                    if (out_popped != nullptr)
                    {
                        out_popped[i] = v;
                    }
                }
                if (i < n && out_ok != nullptr)
                {
                    out_ok[i] = static_cast<uint8_t>(((pushes | pops) >> j) & 1u);
                }
            }
            fence_gpu(); // the element accesses above come before the turns that hand the slots on
#pragma unroll
            for (int j = 0; j < kItems; ++j)
            {
                if (pushes & (1u << j))
                {
                    store_turn_relaxed(seq + pos[j], tk32[j] + 1u);
                }
                else if (pops & (1u << j))
                {
                    store_turn_relaxed(seq + pos[j], tk32[j] + static_cast<unsigned>(cap));
                }
            }
        }
        else
        {
            // One by one in the order of their turns: a push of ticket t before the pop of t, which comes
            // before the push of t + capacity.  Every wait is for a turn that precedes the element's own,
            // so a thread never waits for one of its own later elements (a pop and the push of the same
            // ticket can fall to one thread when the deque runs near empty inside a tile, and a push and
            // the pop one lap earlier when the ring wraps inside a tile).
            unsigned done = 0u;
            const unsigned live = pushes | pops;
#pragma unroll 1
            for (int step = 0; step < kItems; ++step)
            {
                int sel = -1;
                unsigned sel_tk = 0u;
                unsigned sel_pos = 0u;
                bool sel_pop = false;
#pragma unroll
                for (int j = 0; j < kItems; ++j)
                {
                    const bool pj = (pops >> j) & 1u;
                    // order key: ticket, then push before pop (tickets compared modulo 2^32)
                    const bool before = sel < 0 || static_cast<int>(tk32[j] - sel_tk) < 0 ||
                                        (tk32[j] == sel_tk && !pj && sel_pop);
                    if ((((live & ~done) >> j) & 1u) && before)
                    {
                        sel = j;
                        sel_tk = tk32[j];
                        sel_pos = pos[j];
                        sel_pop = pj;
                    }
                }
                if (sel < 0)
                {
                    break;
                }
                done |= 1u << sel;
                const int64_t i = tile + static_cast<int64_t>(sel) * kCThreads + threadIdx.x;
                const unsigned want = sel_pop ? sel_tk + 1u : sel_tk;
                bool ok = false;
                if (wait_turn(seq + sel_pos, want, &c->error))
                {
                    if (sel_pop)
                    {
                        const T v = *reinterpret_cast<volatile T*>(data + sel_pos);
                        store_turn(seq + sel_pos, sel_tk + static_cast<unsigned>(cap));
                        if (out_popped != nullptr)
                        {
                            out_popped[i] = v;
                        }
                    }
                    else
                    {
                        data[sel_pos] = values[i];
                        store_turn(seq + sel_pos, sel_tk + 1u);
                    }
                    ok = true;
                }
                if (out_ok != nullptr)
                {
                    out_ok[i] = static_cast<uint8_t>(ok);
                }
            }
            // elements without a ticket (refused, or past n)
#pragma unroll
            for (int j = 0; j < kItems; ++j)
            {
                const int64_t i = tile + j * kCThreads + threadIdx.x;
                if (!((live >> j) & 1u) && i < n && out_ok != nullptr)
                {
                    out_ok[i] = 0u;
                }
            }
        }
        __syncthreads(); // the counts and reservations are rewritten by the next tile
    }
}

// push_front / pop_back: a launch holds one of them only (the reference runs them concurrently with the
// other end under per-slot locks, src/stdgpu/impl/deque_detail.cuh:260-386).  Element i of the launch acts
// as the i-th of a sequence of calls: push_front of values[0..n) leaves values[n-1] at the front, pop_back
// pops the back element first.  One thread first reserves min(n, room) elements and moves the end
// (k_deque_reserve_end); then element i < k takes ticket t0 - 1 - i.  Nothing else runs on the deque
// during the launch, so there are no slot waits; the slot's turn word is left as the FIFO launches that
// follow expect (a front push leaves the word a push_back of its ticket would leave; a back pop leaves the
// word that lets push_back reuse its ticket).
template <bool FRONT_PUSH>
__global__ void
k_deque_reserve_end(deque_counters* c, int64_t cap, int64_t n)
{
    // push_front needs free capacity (size), pop_back needs elements (avail); both move their end down
    const long long room = FRONT_PUSH ? cap - c->size : c->avail;
    const long long k = room <= 0 ? 0 : (room < n ? room : n);
    unsigned long long* end = FRONT_PUSH ? &c->begin : &c->end;
    c->op_t0 = *end;
    c->op_k = k;
    *end -= static_cast<unsigned long long>(k);
    c->size += FRONT_PUSH ? k : -k;
    c->avail += FRONT_PUSH ? k : -k;
}

template <typename T, bool FRONT_PUSH>
__global__ void
k_deque_end_ops(T* data, unsigned* seq, const deque_counters* c, int64_t cap, const T* values, int64_t n,
                T* out_popped, uint8_t* out_ok)
{
    const unsigned long long t0 = c->op_t0;
    const long long k = c->op_k;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        const bool ok = i < k;
        if (ok)
        {
            const unsigned long long tk = t0 - 1ull - static_cast<unsigned long long>(i);
            const int64_t pos = static_cast<int64_t>(tk % static_cast<unsigned long long>(cap));
            if constexpr (FRONT_PUSH)
            {
                data[pos] = values[i];
                store_turn(seq + pos, static_cast<unsigned>(tk + 1));
            }
            else
            {
                const T v = data[pos];
                store_turn(seq + pos, static_cast<unsigned>(tk));
                if (out_popped != nullptr)
                {
                    out_popped[i] = v;
                }
            }
        }
        if (out_ok != nullptr)
        {
            out_ok[i] = static_cast<uint8_t>(ok);
        }
    }
}

// vector::pop_back for n elements (src/stdgpu/impl/vector_detail.cuh:240-299): element i takes the i-th
// element from the back.  The size is clamped into [0, capacity] first (a push launch may leave it above),
// read by every thread, and lowered by one thread afterwards.
__global__ void
k_vector_clamp(long long* size, int64_t cap, int64_t minus)
{
    long long s = *size;
    s = s < 0 ? 0 : (s > cap ? cap : s);
    s -= minus;
    *size = s < 0 ? 0 : s;
}

// End of every bulk call: size clamped into [0, capacity], the device calls' epoch advanced and the size
// it starts from recorded (sg_vector_sync).
__global__ void
k_vector_epoch(long long* size, int64_t cap, sg_vector_sync* sync, uint32_t epoch)
{
    long long s = *size;
    s = s < 0 ? 0 : (s > cap ? cap : s);
    *size = s;
    sync->base_size = s;
    sync->epoch = epoch;
}

template <typename T>
__global__ void
k_vector_pop_back(const T* data, const long long* size, int64_t n, T* out_values, uint8_t* out_ok)
{
    const long long sz = *size;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        const long long pos = sz - 1 - i;
        const bool ok = pos >= 0;
        if (ok && out_values != nullptr)
        {
            out_values[i] = data[pos];
        }
        if (out_ok != nullptr)
        {
            out_ok[i] = static_cast<uint8_t>(ok);
        }
    }
}

// Before a bulk call: when device calls ran since the last bulk call (they keep per-slot occupied words,
// not turn words), every slot's turn word is rebuilt from the tickets -- a slot holding ticket t (t in
// [begin, end)) gets t + 1, a free slot the ticket of the next push_back that maps to it.
__global__ void
k_deque_rebuild_turns(unsigned* seq, const deque_counters* c, const sg_deque_sync* sync, int64_t cap)
{
    if (*reinterpret_cast<const volatile uint32_t*>(&sync->dirty) == 0u)
    {
        return;
    }
    const unsigned long long b = c->begin;
    const unsigned long long e = c->end;
    const unsigned long long ucap = static_cast<unsigned long long>(cap);
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < cap; i += stride)
    {
        const unsigned long long ui = static_cast<unsigned long long>(i);
        const unsigned long long from_b = (ui + ucap - b % ucap) % ucap; // tickets t = b + from_b map to slot i
        unsigned v;
        if (from_b < e - b)
        {
            v = static_cast<unsigned>(b + from_b + 1ull);
        }
        else
        {
            v = static_cast<unsigned>(e + (ui + ucap - e % ucap) % ucap);
        }
        seq[i] = v;
    }
}

// After the rebuild, and at the end of every bulk call: the device calls' epoch advanced and the tickets
// it starts from recorded; dirty cleared.
__global__ void
k_deque_epoch(const deque_counters* c, sg_deque_sync* sync, uint32_t epoch)
{
    sync->base_begin = c->begin;
    sync->base_end = c->end;
    sync->epoch = epoch;
    sync->dirty = 0u;
}

__global__ void
k_deque_reset(unsigned* seq, deque_counters* c, int64_t cap)
{
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < cap; i += stride)
    {
        seq[i] = static_cast<unsigned>(i);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
    {
        // tickets start at capacity x 2^32: a multiple of the capacity (so ticket mod capacity is the slot)
        // and of 2^32 (so the 32-bit turn words start at the slot index), far enough from zero for
        // push_front to move begin down
        c->size = 0;
        c->begin = static_cast<unsigned long long>(cap) << 32;
        c->end = static_cast<unsigned long long>(cap) << 32;
        c->error = 0;
        c->avail = 0;
    }
}

template <typename T>
__global__ void
k_deque_copy_out(const T* data, const deque_counters* c, int64_t cap, T* out)
{
    const long long n = c->size;
    const unsigned long long b = c->begin;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    for (int64_t i = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        out[i] = data[(b + static_cast<unsigned long long>(i)) % static_cast<unsigned long long>(cap)];
    }
}

// ---------------------------------------------------------------- bitset::count

constexpr int kCountThreads = 512;

__global__ void __launch_bounds__(kCountThreads)
k_bitset_count(const uint32_t* blocks, int64_t nbits, unsigned long long* partials)
{
    const int64_t nwords = (nbits + 31) / 32;
    const int64_t full_words = nbits / 32; // words with all 32 bits counted
    const bool aligned = (reinterpret_cast<uintptr_t>(blocks) & 15u) == 0;
    const int64_t nvec = aligned ? full_words / 4 : 0;
    const int64_t tid = blockIdx.x * static_cast<int64_t>(blockDim.x) + threadIdx.x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    unsigned long long sum = 0;
    const uint4* v4 = reinterpret_cast<const uint4*>(blocks);
    // 4 independent 16-byte loads in flight per thread
    int64_t k = tid;
    for (; k + 3 * stride < nvec; k += 4 * stride)
    {
        const uint4 a = __ldcs(v4 + k);
        const uint4 b = __ldcs(v4 + k + stride);
        const uint4 c = __ldcs(v4 + k + 2 * stride);
        const uint4 d = __ldcs(v4 + k + 3 * stride);
        sum += __popc(a.x) + __popc(a.y) + __popc(a.z) + __popc(a.w);
        sum += __popc(b.x) + __popc(b.y) + __popc(b.z) + __popc(b.w);
        sum += __popc(c.x) + __popc(c.y) + __popc(c.z) + __popc(c.w);
        sum += __popc(d.x) + __popc(d.y) + __popc(d.z) + __popc(d.w);
    }
    for (; k < nvec; k += stride)
    {
        const uint4 a = __ldcs(v4 + k);
        sum += __popc(a.x) + __popc(a.y) + __popc(a.z) + __popc(a.w);
    }
    // remaining full words, then the masked tail word (count_block_bits::block_mask)
    for (int64_t w = nvec * 4 + tid; w < nwords; w += stride)
    {
        uint32_t x = blocks[w];
        if (w >= full_words)
        {
            const int rem = static_cast<int>(nbits - w * 32);
            x &= (1u << rem) - 1u;
        }
        sum += __popc(x);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
    }
    __shared__ unsigned long long red[kCountThreads / 32];
    if ((threadIdx.x & 31) == 0)
    {
        red[threadIdx.x >> 5] = sum;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        unsigned long long s = 0;
        for (int w = 0; w < kCountThreads / 32; ++w)
        {
            s += red[w];
        }
        partials[blockIdx.x] = s;
    }
}

__global__ void __launch_bounds__(1024)
k_sum_partials(const unsigned long long* partials, int n, unsigned long long* out)
{
    unsigned long long s = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x)
    {
        s += partials[i];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        s += __shfl_xor_sync(0xffffffffu, s, o);
    }
    __shared__ unsigned long long red[32];
    if ((threadIdx.x & 31) == 0)
    {
        red[threadIdx.x >> 5] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        unsigned long long t = 0;
        for (int w = 0; w < static_cast<int>(blockDim.x >> 5); ++w)
        {
            t += red[w];
        }
        *out = t;
    }
}

int
count_grid()
{
    static const int g = persistent_grid(k_bitset_count, kCountThreads);
    return g;
}

// ---------------------------------------------------------------- allocation-free bitset::count
// The same count with its scratch in a fixed array compiled into the library instead of memory the
// library allocates: one partial sum per CTA, each CTA owning a fixed chunk of the blocks, so the
// array's length bounds the largest input.  The array lives in every GPU that loads the library until
// the process exits; all calls on a device share it, so calls that overlap on the GPU race.

constexpr int kNoAllocPartials = 8192;                                   // 64 KiB of partial sums
constexpr int64_t kNoAllocChunkWords = 65536;                            // 32-bit blocks per CTA (256 KiB)
constexpr int64_t kNoAllocMaxBits = kNoAllocPartials * kNoAllocChunkWords * 32; // 2^34 bits

static __device__ __align__(256) unsigned long long g_noalloc_partials[kNoAllocPartials];

__global__ void __launch_bounds__(kCountThreads)
k_bitset_count_chunked(const uint32_t* blocks, int64_t nbits, unsigned long long* partials)
{
    const int64_t nwords = (nbits + 31) / 32;
    const int64_t full_words = nbits / 32;
    const int64_t lo = static_cast<int64_t>(blockIdx.x) * kNoAllocChunkWords;
    const int64_t hi = lo + kNoAllocChunkWords < nwords ? lo + kNoAllocChunkWords : nwords;
    unsigned long long sum = 0;
    const bool aligned = (reinterpret_cast<uintptr_t>(blocks) & 15u) == 0;
    int64_t w = lo;
    if (aligned)
    {
        // whole 16-byte vectors of full words inside the chunk
        const int64_t vhi = lo + ((min(hi, full_words) - lo) / 4) * 4;
        const uint4* v4 = reinterpret_cast<const uint4*>(blocks + lo);
        const int64_t nv = (vhi - lo) / 4;
        for (int64_t k = threadIdx.x; k < nv; k += blockDim.x)
        {
            const uint4 a = __ldcs(v4 + k);
            sum += __popc(a.x) + __popc(a.y) + __popc(a.z) + __popc(a.w);
        }
        w = vhi;
    }
    for (int64_t x = w + threadIdx.x; x < hi; x += blockDim.x)
    {
        uint32_t b = blocks[x];
        if (x >= full_words)
        {
            b &= (1u << static_cast<int>(nbits - x * 32)) - 1u;
        }
        sum += __popc(b);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
    {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
    }
    __shared__ unsigned long long red[kCountThreads / 32];
    if ((threadIdx.x & 31) == 0)
    {
        red[threadIdx.x >> 5] = sum;
    }
    __syncthreads();
    if (threadIdx.x == 0)
    {
        unsigned long long t = 0;
        for (int k = 0; k < kCountThreads / 32; ++k)
        {
            t += red[k];
        }
        partials[blockIdx.x] = t; // every entry the sum kernel reads is written by this call
    }
}

} // namespace detail
} // namespace sg

using namespace sg::detail;

struct sg_vector
{
    int32_t elem_bytes;
    int64_t capacity;
    void* data;
    long long* size;
    long long* host;
    uint16_t* slot_state;   // device calls' per-slot words (sg_vector_sync)
    sg_vector_sync* sync;
    uint32_t epoch;         // host copy of sync->epoch
    object_allocator oa;            // the vector's own allocator (sg_vector_create_with_allocator), or none
    void (*release_ctx)(void* ctx); // called with oa.ctx when the vector is destroyed (nullable)
};

struct sg_deque
{
    int32_t elem_bytes;
    int64_t capacity;
    void* data;
    unsigned* seq;
    deque_counters* counters;
    deque_counters* host;
    uint16_t* slot_state; // device calls' per-slot words (sg_deque_sync)
    sg_deque_sync* sync;
    uint32_t epoch;       // host copy of sync->epoch
    object_allocator oa;            // the deque's own allocator (sg_deque_create_with_allocator), or none
    void (*release_ctx)(void* ctx); // called with oa.ctx when the deque is destroyed (nullable)
};

namespace
{

// Per-device scratch of bitset::count: one partial per block plus the result word.
struct count_scratch
{
    unsigned long long* partials = nullptr;
    unsigned long long* host = nullptr;
    int blocks = 0;
};

std::mutex g_count_mutex;
count_scratch g_count_scratch[64];

} // namespace

namespace
{

// Every bulk call on a deque runs between these two: the turn words rebuilt if device calls ran since the
// last bulk call, and afterwards the device calls' epoch advanced (slot words cleared when it wraps).
sg_status
deque_bulk_begin(sg_deque* d, cudaStream_t s)
{
    static const int mg = persistent_grid(k_deque_rebuild_turns, kCThreads);
    k_deque_rebuild_turns<<<grid_for(d->capacity, kCThreads, mg), kCThreads, 0, s>>>(d->seq, d->counters, d->sync,
                                                                                     d->capacity);
    SG_LAUNCH_CHECK();
    return SG_OK;
}

sg_status
deque_bulk_end(sg_deque* d, cudaStream_t s)
{
    uint32_t e = d->epoch + 1;
    if (e > 32767u)
    {
        SG_CUDA_TRY(cudaMemsetAsync(d->slot_state, 0, static_cast<size_t>(d->capacity) * sizeof(uint16_t), s));
        e = 1;
    }
    d->epoch = e;
    k_deque_epoch<<<1, 1, 0, s>>>(d->counters, d->sync, e);
    SG_LAUNCH_CHECK();
    return SG_OK;
}

template <bool FRONT_PUSH>
sg_status
deque_end_ops(sg_deque* d, const void* values, int64_t n, void* out_popped, uint8_t* out_ok, void* stream)
{
    if (d == nullptr || n < 0 || (FRONT_PUSH && n > 0 && values == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    cudaStream_t s = as_stream(stream);
    sg_status st = deque_bulk_begin(d, s);
    if (st != SG_OK)
    {
        return st;
    }
    k_deque_reserve_end<FRONT_PUSH><<<1, 1, 0, s>>>(d->counters, d->capacity, n);
    SG_LAUNCH_CHECK();
    const int g = grid_for(n, kCThreads, 4096);
    if (d->elem_bytes == 4)
    {
        k_deque_end_ops<uint32_t, FRONT_PUSH><<<g, kCThreads, 0, s>>>(
                static_cast<uint32_t*>(d->data), d->seq, d->counters, d->capacity, static_cast<const uint32_t*>(values), n,
                static_cast<uint32_t*>(out_popped), out_ok);
    }
    else
    {
        k_deque_end_ops<unsigned long long, FRONT_PUSH><<<g, kCThreads, 0, s>>>(
                static_cast<unsigned long long*>(d->data), d->seq, d->counters, d->capacity,
                static_cast<const unsigned long long*>(values), n, static_cast<unsigned long long*>(out_popped), out_ok);
    }
    SG_LAUNCH_CHECK();
    return deque_bulk_end(d, s);
}

} // namespace

namespace
{

// Ends a bulk call on v: the next epoch (1 .. 32767; slot words are cleared when it wraps).
sg_status
vector_next_epoch(sg_vector* v, cudaStream_t s)
{
    uint32_t e = v->epoch + 1;
    if (e > 32767u)
    {
        SG_CUDA_TRY(cudaMemsetAsync(v->slot_state, 0, static_cast<size_t>(v->capacity) * sizeof(uint16_t), s));
        e = 1;
    }
    v->epoch = e;
    k_vector_epoch<<<1, 1, 0, s>>>(v->size, v->capacity, v->sync, e);
    SG_LAUNCH_CHECK();
    return SG_OK;
}

} // namespace

extern "C" {

static sg_status
create_vector(int32_t elem_bytes, int64_t capacity, const object_allocator& oa, sg_vector** out)
{
    if (out == nullptr || (elem_bytes != 4 && elem_bytes != 8) || capacity <= 0)
    {
        return SG_ERR_BAD_ARG;
    }
    *out = nullptr;
    auto* v = new (std::nothrow) sg_vector{};
    if (v == nullptr)
    {
        return SG_ERR_OOM;
    }
    v->elem_bytes = elem_bytes;
    v->capacity = capacity;
    v->oa = oa;
    cudaError_t e = sg::detail::obj_malloc(v->oa, &v->data, static_cast<size_t>(capacity) * elem_bytes);
    if (e == cudaSuccess)
    {
        e = sg::detail::obj_malloc(v->oa, &v->size, sizeof(long long));
    }
    if (e == cudaSuccess)
    {
        e = cudaMemset(v->size, 0, sizeof(long long));
    }
    if (e == cudaSuccess)
    {
        e = cudaMallocHost(&v->host, sizeof(long long));
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::obj_malloc(v->oa, &v->slot_state, static_cast<size_t>(capacity) * sizeof(uint16_t));
    }
    if (e == cudaSuccess)
    {
        e = cudaMemset(v->slot_state, 0, static_cast<size_t>(capacity) * sizeof(uint16_t));
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::obj_malloc(v->oa, &v->sync, sizeof(sg_vector_sync));
    }
    if (e == cudaSuccess)
    {
        const sg_vector_sync init{ 1u, 0u, 0 };
        v->epoch = 1;
        e = cudaMemcpy(v->sync, &init, sizeof(init), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess)
    {
        sg_vector_destroy(v);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA;
    }
    *out = v;
    return SG_OK;
}

sg_status
sg_vector_create(int32_t elem_bytes, int64_t capacity, sg_vector** out)
{
    return create_vector(elem_bytes, capacity, object_allocator{}, out);
}

sg_status
sg_vector_create_with_allocator(int32_t elem_bytes, int64_t capacity, const sg_allocator* allocator, sg_vector** out)
{
    if (allocator == nullptr || allocator->alloc == nullptr || allocator->release == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    const sg_status st =
            create_vector(elem_bytes, capacity, object_allocator{ allocator->alloc, allocator->release, allocator->ctx }, out);
    if (st == SG_OK)
    {
        (*out)->release_ctx = allocator->release_ctx;
    }
    return st;
}

sg_status
sg_vector_destroy(sg_vector* v)
{
    if (v == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaDeviceSynchronize();
    sg::detail::obj_free(v->oa, v->data);
    sg::detail::obj_free(v->oa, v->size);
    sg::detail::obj_free(v->oa, v->slot_state);
    sg::detail::obj_free(v->oa, v->sync);
    if (v->host != nullptr)
    {
        cudaFreeHost(v->host);
    }
    if (v->release_ctx != nullptr)
    {
        v->release_ctx(v->oa.ctx);
    }
    delete v;
    return SG_OK;
}

sg_status
sg_vector_push_back(sg_vector* v, const void* values, const uint8_t* pred, int64_t n, uint8_t* out_pushed,
                    void* stream)
{
    if (v == nullptr || n < 0 || (n > 0 && values == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    cudaStream_t s = as_stream(stream);
    if (v->elem_bytes == 4)
    {
        static const int mg = persistent_grid(k_vector_push_back<uint32_t>, kCThreads);
        k_vector_push_back<uint32_t><<<grid_for(n, static_cast<int>(kVecTileElems), mg), kCThreads, 0, s>>>(
                static_cast<uint32_t*>(v->data), v->size, v->capacity, static_cast<const uint32_t*>(values), pred, n,
                out_pushed);
    }
    else
    {
        static const int mg = persistent_grid(k_vector_push_back<unsigned long long>, kCThreads);
        k_vector_push_back<unsigned long long><<<grid_for(n, static_cast<int>(kVecTileElems), mg), kCThreads, 0, s>>>(
                static_cast<unsigned long long*>(v->data), v->size, v->capacity,
                static_cast<const unsigned long long*>(values), pred, n, out_pushed);
    }
    SG_LAUNCH_CHECK();
    return vector_next_epoch(v, s);
}

sg_status
sg_vector_size(sg_vector* v, void* stream, int64_t* out_size)
{
    if (v == nullptr || out_size == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = as_stream(stream);
    SG_CUDA_TRY(cudaMemcpyAsync(v->host, v->size, sizeof(long long), cudaMemcpyDeviceToHost, s));
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    long long x = *v->host;
    *out_size = x < 0 ? 0 : (x > v->capacity ? v->capacity : x);
    return SG_OK;
}

sg_status
sg_vector_clear(sg_vector* v, void* stream)
{
    if (v == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    SG_CUDA_TRY(cudaMemsetAsync(v->size, 0, sizeof(long long), as_stream(stream)));
    return vector_next_epoch(v, as_stream(stream));
}

sg_status
sg_vector_pop_back(sg_vector* v, int64_t n, void* out_values, uint8_t* out_ok, void* stream)
{
    if (v == nullptr || n < 0)
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    cudaStream_t s = as_stream(stream);
    k_vector_clamp<<<1, 1, 0, s>>>(v->size, v->capacity, 0);
    SG_LAUNCH_CHECK();
    const int g = grid_for(n, kCThreads, 4096);
    if (v->elem_bytes == 4)
    {
        k_vector_pop_back<uint32_t><<<g, kCThreads, 0, s>>>(static_cast<const uint32_t*>(v->data), v->size, n,
                                                            static_cast<uint32_t*>(out_values), out_ok);
    }
    else
    {
        k_vector_pop_back<unsigned long long><<<g, kCThreads, 0, s>>>(
                static_cast<const unsigned long long*>(v->data), v->size, n, static_cast<unsigned long long*>(out_values),
                out_ok);
    }
    SG_LAUNCH_CHECK();
    k_vector_clamp<<<1, 1, 0, s>>>(v->size, v->capacity, n);
    SG_LAUNCH_CHECK();
    return vector_next_epoch(v, s);
}

sg_status
sg_vector_insert(sg_vector* v, const void* values, int64_t n, void* stream)
{
    if (v == nullptr || n < 0 || (n > 0 && values == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    int64_t size = 0;
    const sg_status st = sg_vector_size(v, stream, &size);
    if (st != SG_OK)
    {
        return st;
    }
    if (size + n > v->capacity)
    {
        return SG_ERR_FULL; // nothing inserted (vector_detail.cuh:372-410 refuses the whole range)
    }
    cudaStream_t s = as_stream(stream);
    SG_CUDA_TRY(cudaMemcpyAsync(static_cast<char*>(v->data) + size * v->elem_bytes, values,
                                static_cast<size_t>(n) * v->elem_bytes, cudaMemcpyDeviceToDevice, s));
    *v->host = size + n;
    SG_CUDA_TRY(cudaMemcpyAsync(v->size, v->host, sizeof(long long), cudaMemcpyHostToDevice, s));
    const sg_status e = vector_next_epoch(v, s);
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    return e;
}

sg_status
sg_vector_erase(sg_vector* v, int64_t n, void* stream)
{
    if (v == nullptr || n < 0)
    {
        return SG_ERR_BAD_ARG;
    }
    int64_t size = 0;
    const sg_status st = sg_vector_size(v, stream, &size);
    if (st != SG_OK)
    {
        return st;
    }
    if (n > size)
    {
        return SG_ERR_BAD_ARG; // nothing erased (vector_detail.cuh:418-450 refuses a range past the start)
    }
    cudaStream_t s = as_stream(stream);
    *v->host = size - n;
    SG_CUDA_TRY(cudaMemcpyAsync(v->size, v->host, sizeof(long long), cudaMemcpyHostToDevice, s));
    const sg_status e = vector_next_epoch(v, s);
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    return e;
}

sg_status
sg_vector_view_of(const sg_vector* v, sg_vector_view* out)
{
    if (v == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    out->data = v->data;
    out->size = v->size;
    out->capacity = v->capacity;
    out->elem_bytes = v->elem_bytes;
    out->pad = 0;
    out->slot_state = v->slot_state;
    out->sync = v->sync;
    return SG_OK;
}

static sg_status
create_deque(int32_t elem_bytes, int64_t capacity, const object_allocator& oa, sg_deque** out)
{
    if (out == nullptr || (elem_bytes != 4 && elem_bytes != 8) || capacity <= 0 || capacity >= (int64_t{ 1 } << 31))
    {
        return SG_ERR_BAD_ARG;
    }
    *out = nullptr;
    auto* d = new (std::nothrow) sg_deque{};
    if (d == nullptr)
    {
        return SG_ERR_OOM;
    }
    d->elem_bytes = elem_bytes;
    d->capacity = capacity;
    d->oa = oa;
    cudaError_t e = sg::detail::obj_malloc(d->oa, &d->data, static_cast<size_t>(capacity) * elem_bytes);
    if (e == cudaSuccess)
    {
        e = sg::detail::obj_malloc(d->oa, &d->seq, static_cast<size_t>(capacity) * sizeof(unsigned));
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::obj_malloc(d->oa, &d->counters, sizeof(deque_counters));
    }
    if (e == cudaSuccess)
    {
        e = cudaMallocHost(&d->host, sizeof(deque_counters));
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::obj_malloc(d->oa, &d->slot_state, static_cast<size_t>(capacity) * sizeof(uint16_t));
    }
    if (e == cudaSuccess)
    {
        e = cudaMemset(d->slot_state, 0, static_cast<size_t>(capacity) * sizeof(uint16_t));
    }
    if (e == cudaSuccess)
    {
        e = sg::detail::obj_malloc(d->oa, &d->sync, sizeof(sg_deque_sync));
    }
    if (e == cudaSuccess)
    {
        e = cudaMemset(d->sync, 0, sizeof(sg_deque_sync));
    }
    if (e != cudaSuccess)
    {
        sg_deque_destroy(d);
        cudaGetLastError();
        return e == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA;
    }
    sg_status st = sg_deque_clear(d, nullptr);
    if (st != SG_OK)
    {
        sg_deque_destroy(d);
        return st;
    }
    *out = d;
    return SG_OK;
}

sg_status
sg_deque_create(int32_t elem_bytes, int64_t capacity, sg_deque** out)
{
    return create_deque(elem_bytes, capacity, object_allocator{}, out);
}

sg_status
sg_deque_create_with_allocator(int32_t elem_bytes, int64_t capacity, const sg_allocator* allocator, sg_deque** out)
{
    if (allocator == nullptr || allocator->alloc == nullptr || allocator->release == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    const sg_status st =
            create_deque(elem_bytes, capacity, object_allocator{ allocator->alloc, allocator->release, allocator->ctx }, out);
    if (st == SG_OK)
    {
        (*out)->release_ctx = allocator->release_ctx;
    }
    return st;
}

sg_status
sg_deque_destroy(sg_deque* d)
{
    if (d == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaDeviceSynchronize();
    sg::detail::obj_free(d->oa, d->data);
    sg::detail::obj_free(d->oa, d->seq);
    sg::detail::obj_free(d->oa, d->counters);
    sg::detail::obj_free(d->oa, d->slot_state);
    sg::detail::obj_free(d->oa, d->sync);
    if (d->host != nullptr)
    {
        cudaFreeHost(d->host);
    }
    if (d->release_ctx != nullptr)
    {
        d->release_ctx(d->oa.ctx);
    }
    delete d;
    return SG_OK;
}

sg_status
sg_deque_clear(sg_deque* d, void* stream)
{
    if (d == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = as_stream(stream);
    static const int mg = persistent_grid(k_deque_reset, kCThreads);
    k_deque_reset<<<grid_for(d->capacity, kCThreads, mg), kCThreads, 0, s>>>(d->seq, d->counters, d->capacity);
    SG_LAUNCH_CHECK();
    return deque_bulk_end(d, s);
}

sg_status
sg_deque_push_front(sg_deque* d, const void* values, int64_t n, uint8_t* out_ok, void* stream)
{
    return deque_end_ops<true>(d, values, n, nullptr, out_ok, stream);
}

sg_status
sg_deque_pop_back(sg_deque* d, int64_t n, void* out_popped, uint8_t* out_ok, void* stream)
{
    return deque_end_ops<false>(d, nullptr, n, out_popped, out_ok, stream);
}

sg_status
sg_deque_ops(sg_deque* d, const uint8_t* is_push, const void* values, int64_t n, void* out_popped, uint8_t* out_ok,
             void* stream)
{
    if (d == nullptr || n < 0)
    {
        return SG_ERR_BAD_ARG;
    }
    if (n == 0)
    {
        return SG_OK;
    }
    cudaStream_t s = as_stream(stream);
    sg_status st = deque_bulk_begin(d, s);
    if (st != SG_OK)
    {
        return st;
    }
    if (d->elem_bytes == 4)
    {
        static const int mg = persistent_grid(k_deque_ops<uint32_t>, kCThreads);
        k_deque_ops<uint32_t><<<grid_for(n, static_cast<int>(kTileElems), mg), kCThreads, 0, s>>>(
                static_cast<uint32_t*>(d->data), d->seq, d->counters, d->capacity, is_push,
                static_cast<const uint32_t*>(values), n, static_cast<uint32_t*>(out_popped), out_ok);
    }
    else
    {
        static const int mg = persistent_grid(k_deque_ops<unsigned long long>, kCThreads);
        k_deque_ops<unsigned long long><<<grid_for(n, static_cast<int>(kTileElems), mg), kCThreads, 0, s>>>(
                static_cast<unsigned long long*>(d->data), d->seq, d->counters, d->capacity, is_push,
                static_cast<const unsigned long long*>(values), n, static_cast<unsigned long long*>(out_popped),
                out_ok);
    }
    SG_LAUNCH_CHECK();
    return deque_bulk_end(d, s);
}

sg_status
sg_deque_size(sg_deque* d, void* stream, int64_t* out_size)
{
    if (d == nullptr || out_size == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = as_stream(stream);
    SG_CUDA_TRY(cudaMemcpyAsync(d->host, d->counters, sizeof(deque_counters), cudaMemcpyDeviceToHost, s));
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    const long long x = d->host->size;
    *out_size = x < 0 ? 0 : (x > d->capacity ? d->capacity : x);
    return (d->host->error & kDequeErrWait) != 0u ? SG_ERR_RETRY_EXHAUSTED : SG_OK;
}

sg_status
sg_deque_copy_out(sg_deque* d, void* out, void* stream, int64_t* out_n)
{
    if (d == nullptr || out == nullptr || out_n == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    cudaStream_t s = as_stream(stream);
    int64_t n = 0;
    sg_status st = sg_deque_size(d, stream, &n);
    if (st != SG_OK)
    {
        return st;
    }
    if (n > 0)
    {
        const int grid = grid_for(n, kCThreads, 4096);
        if (d->elem_bytes == 4)
        {
            k_deque_copy_out<uint32_t><<<grid, kCThreads, 0, s>>>(static_cast<const uint32_t*>(d->data), d->counters,
                                                                  d->capacity, static_cast<uint32_t*>(out));
        }
        else
        {
            k_deque_copy_out<unsigned long long><<<grid, kCThreads, 0, s>>>(
                    static_cast<const unsigned long long*>(d->data), d->counters, d->capacity,
                    static_cast<unsigned long long*>(out));
        }
        SG_LAUNCH_CHECK();
        SG_CUDA_TRY(cudaStreamSynchronize(s));
    }
    *out_n = n;
    return SG_OK;
}

sg_status
sg_deque_view_of(const sg_deque* d, sg_deque_view* out)
{
    if (d == nullptr || out == nullptr)
    {
        return SG_ERR_BAD_ARG;
    }
    out->data = d->data;
    out->seq = d->seq;
    out->counters = d->counters;
    out->capacity = d->capacity;
    out->elem_bytes = d->elem_bytes;
    out->pad = 0;
    out->slot_state = d->slot_state;
    out->sync = d->sync;
    return SG_OK;
}

sg_status
sg_bitset_count(const uint32_t* blocks, int64_t nbits, void* stream, int64_t* out_count)
{
    if (out_count == nullptr || nbits < 0 || (nbits > 0 && blocks == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    if (nbits == 0)
    {
        *out_count = 0;
        return SG_OK;
    }
    int dev = 0;
    SG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64)
    {
        return SG_ERR_NO_DEVICE;
    }
    cudaStream_t s = as_stream(stream);
    std::lock_guard<std::mutex> lock(g_count_mutex);
    count_scratch& sc = g_count_scratch[dev];
    if (sc.partials == nullptr)
    {
        const int blocks_max = count_grid();
        SG_CUDA_TRY(cudaMalloc(&sc.partials, static_cast<size_t>(blocks_max + 1) * sizeof(unsigned long long)));
        SG_CUDA_TRY(cudaMallocHost(&sc.host, sizeof(unsigned long long)));
        sc.blocks = blocks_max;
    }
    const int64_t nvec = (nbits + 127) / 128;
    const int grid = grid_for(nvec, kCountThreads * 4, sc.blocks);
    k_bitset_count<<<grid, kCountThreads, 0, s>>>(blocks, nbits, sc.partials);
    SG_LAUNCH_CHECK();
    k_sum_partials<<<1, 1024, 0, s>>>(sc.partials, grid, sc.partials + sc.blocks);
    SG_LAUNCH_CHECK();
    SG_CUDA_TRY(cudaMemcpyAsync(sc.host, sc.partials + sc.blocks, sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                                s));
    SG_CUDA_TRY(cudaStreamSynchronize(s));
    *out_count = static_cast<int64_t>(*sc.host);
    return SG_OK;
}

} // extern "C"

namespace
{

// Device address of the fixed scratch array, looked up once per device with that device current.
std::mutex g_noalloc_mutex;
unsigned long long* g_noalloc_ptr[64] = {};

sg_status
noalloc_scratch(unsigned long long** out)
{
    int dev = 0;
    SG_CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64)
    {
        return SG_ERR_NO_DEVICE;
    }
    std::lock_guard<std::mutex> lock(g_noalloc_mutex);
    if (g_noalloc_ptr[dev] == nullptr)
    {
        void* p = nullptr;
        // the symbol name in host code is a host-side stand-in; the kernels need its device address
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_partials);
        if (e != cudaSuccess || p == nullptr)
        {
            cudaGetLastError();
            return SG_ERR_CUDA;
        }
        g_noalloc_ptr[dev] = static_cast<unsigned long long*>(p);
    }
    *out = g_noalloc_ptr[dev];
    return SG_OK;
}

} // namespace

extern "C" {

sg_status
sg_bitset_count_noalloc(const uint32_t* blocks, int64_t nbits, int64_t* out_count, void* stream)
{
    if (out_count == nullptr || nbits < 0 || (nbits > 0 && blocks == nullptr))
    {
        return SG_ERR_BAD_ARG;
    }
    if (nbits > kNoAllocMaxBits)
    {
        return SG_ERR_BAD_ARG; // more chunks than the fixed scratch array holds partial sums for
    }
    unsigned long long* scratch = nullptr;
    sg_status st = noalloc_scratch(&scratch);
    if (st != SG_OK)
    {
        return st;
    }
    cudaStream_t s = as_stream(stream);
    const int64_t nwords = (nbits + 31) / 32;
    const int chunks = static_cast<int>((nwords + kNoAllocChunkWords - 1) / kNoAllocChunkWords);
    if (chunks > 0)
    {
        k_bitset_count_chunked<<<chunks, kCountThreads, 0, s>>>(blocks, nbits, scratch);
        SG_LAUNCH_CHECK();
    }
    k_sum_partials<<<1, 1024, 0, s>>>(scratch, chunks, reinterpret_cast<unsigned long long*>(out_count));
    SG_LAUNCH_CHECK();
    return SG_OK;
}

} // extern "C"

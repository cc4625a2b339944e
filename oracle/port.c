/*
 * Oracle restatement (test infrastructure only): see port.h.
 *
 * Reference: stdgpu 1.3.0.  Paths are relative to the reference project root.
 * The table keeps the reference layout -- bucket_count home slots followed by
 * excess_count overflow slots, chains linked by relative offsets, an occupied
 * flag per slot, a global occupied count and an excess free-list vector -- so
 * that refusal (full table, empty excess list), geometry and bucket() answers
 * follow the reference exactly.
 */
#include "port.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

struct port_table
{
    int64_t bucket_count;
    int64_t excess_count;
    int64_t total_count;
    uint64_t* keys;    /* _values (key part)   unordered_base.cuh */
    uint64_t* vals;    /* _values (mapped part) */
    uint64_t* hashes;  /* Hash(key) of each slot's key (the identity for integer keys) */
    int64_t* offsets;  /* _offsets: relative link to the next chain entry, 0 = end */
    uint8_t* occupied; /* _occupied bitset, one byte per slot here */
    int64_t occupied_count; /* _occupied_count */
    int64_t* excess;   /* _excess_list_positions data */
    int64_t excess_size;
};

/* bit_width / bit_ceil: src/stdgpu/impl/bit_detail.h:36-62, 94-113 */
static uint64_t bit_width_u64(uint64_t x)
{
    uint64_t r = 0;
    while (x)
    {
        ++r;
        x >>= 1;
    }
    return r;
}

static uint64_t bit_ceil_u64(uint64_t x)
{
    uint64_t r = 1;
    if (x <= 1)
        return 1;
    while (r < x && r != 0)
        r <<= 1;
    return r;
}

/* src/stdgpu/impl/unordered_base_detail.cuh:56-85 */
int64_t port_fibonacci_hashing(uint64_t hash, int64_t bucket_count)
{
    int64_t max_bit_width_result = (int64_t)bit_width_u64((uint64_t)bucket_count) - 1;
    if (max_bit_width_result <= 0)
        return 0;
    uint64_t dropped = (uint64_t)(64 - max_bit_width_result);
    uint64_t improved = hash ^ (hash >> dropped);
    const uint64_t multiplier = 11400714819323198485ULL; /* 2^64 / golden ratio */
    return (int64_t)((multiplier * improved) >> dropped);
}

/* src/stdgpu/impl/unordered_base_detail.cuh:34-48 (long double, as the reference) */
int64_t port_expected_collisions(int64_t bucket_count, int64_t capacity)
{
    long double k = (long double)bucket_count;
    long double n = (long double)capacity;
    return (int64_t)ceill(n * (1.0L - powl(1.0L - (1.0L / k), n - 1.0L)));
}

/* src/stdgpu/impl/unordered_base_detail.cuh:1264-1273: the capacity passes through float */
void port_geometry(int64_t capacity, int64_t* bucket_count, int64_t* excess_count, int64_t* total_count)
{
    float c = ceilf((float)capacity / 1.0F); /* default_max_load_factor() == 1.0F (:50-54) */
    int64_t b = (int64_t)bit_ceil_u64((uint64_t)c);
    int64_t e = port_expected_collisions(b, capacity) + 1;
    *bucket_count = b;
    *excess_count = e;
    *total_count = b + e;
}

/* vector_clear_iota(excess, bucket_count): src/stdgpu/impl/vector_detail.cuh:361-368 */
static void reset_excess(port_table* t)
{
    for (int64_t i = 0; i < t->excess_count; ++i)
        t->excess[i] = t->bucket_count + i;
    t->excess_size = t->excess_count;
}

/* createDeviceObject: src/stdgpu/impl/unordered_base_detail.cuh:1254-1308 */
port_table* port_create(int64_t capacity)
{
    port_table* t = (port_table*)calloc(1, sizeof(port_table));
    port_geometry(capacity, &t->bucket_count, &t->excess_count, &t->total_count);
    size_t n = (size_t)t->total_count;
    t->keys = (uint64_t*)calloc(n, sizeof(uint64_t));
    t->vals = (uint64_t*)calloc(n, sizeof(uint64_t));
    t->offsets = (int64_t*)calloc(n, sizeof(int64_t));
    t->hashes = (uint64_t*)calloc(n, sizeof(uint64_t));
    t->occupied = (uint8_t*)calloc(n, 1);
    t->excess = (int64_t*)calloc((size_t)t->excess_count, sizeof(int64_t));
    t->occupied_count = 0;
    reset_excess(t);
    return t;
}

/* destroyDeviceObject: src/stdgpu/impl/unordered_base_detail.cuh:1310-1348 */
void port_destroy(port_table* t)
{
    if (!t)
        return;
    free(t->keys);
    free(t->vals);
    free(t->hashes);
    free(t->offsets);
    free(t->occupied);
    free(t->excess);
    free(t);
}

/* bucket / bucket_impl: src/stdgpu/impl/unordered_base_detail.cuh:547-564 with hash<integral> = identity
 * (src/stdgpu/impl/functional_detail.h:60-80) */
int64_t port_bucket(const port_table* t, uint64_t key)
{
    return port_fibonacci_hashing(key, t->bucket_count);
}

/* find_impl: src/stdgpu/impl/unordered_base_detail.cuh:653-682; returns the slot or -1 (end()).
 * hash: Hash(key), whose fibonacci hashing is the key's bucket (bucket_impl :547-564). */
static int64_t find_pos_h(const port_table* t, uint64_t key, uint64_t hash)
{
    int64_t i = port_fibonacci_hashing(hash, t->bucket_count);
    if (t->occupied[i] && t->keys[i] == key)
        return i;
    while (t->offsets[i] != 0)
    {
        i += t->offsets[i];
        if (t->occupied[i] && t->keys[i] == key)
            return i;
    }
    return -1;
}

static int64_t find_pos(const port_table* t, uint64_t key)
{
    return find_pos_h(t, key, key);
}

int port_find_h(const port_table* t, uint64_t key, uint64_t hash, uint64_t* value)
{
    int64_t p = find_pos_h(t, key, hash);
    if (p < 0)
        return 0;
    if (value)
        *value = t->vals[p];
    return 1;
}

int port_find(const port_table* t, uint64_t key, uint64_t* value)
{
    int64_t p = find_pos(t, key);
    if (p < 0)
        return 0;
    if (value)
        *value = t->vals[p];
    return 1;
}

/* find_linked_list_end: src/stdgpu/impl/unordered_base_detail.cuh:915-928 */
static int64_t find_linked_list_end(const port_table* t, int64_t start)
{
    int64_t e = start;
    while (t->offsets[e] != 0)
        e += t->offsets[e];
    return e;
}

/* find_previous_entry_position: src/stdgpu/impl/unordered_base_detail.cuh:930-956 */
static int64_t find_previous_entry_position(const port_table* t, int64_t entry, int64_t start)
{
    int64_t prev = start;
    int64_t i = start;
    while (t->offsets[i] != 0)
    {
        i += t->offsets[i];
        if (i == entry)
            break;
        prev = i;
    }
    return prev;
}

/* full(): src/stdgpu/impl/unordered_base_detail.cuh:1094-1099 */
static int is_full(const port_table* t)
{
    return t->occupied_count == t->total_count;
}

/* insert(value) retry loop :967-994 around try_insert :708-809, run by one thread */
int port_insert_h(port_table* t, uint64_t key, uint64_t hash, uint64_t value)
{
    /* loop guard :980-981: refuse when full or when the excess free-list is empty */
    if (is_full(t) || t->excess_size == 0)
        return 0;
    /* :719 / :803-806 the key is present: no action */
    if (find_pos_h(t, key, hash) >= 0)
        return 0;
    int64_t b = port_fibonacci_hashing(hash, t->bucket_count);
    if (!t->occupied[b])
    {
        /* :723-753 free bucket: construct in place, the chain link is left untouched */
        t->keys[b] = key;
        t->vals[b] = value;
        t->hashes[b] = hash;
        ++t->occupied_count;
        t->occupied[b] = 1;
        return 1;
    }
    /* :754-801 append to the chain end with a slot popped from the excess list */
    int64_t end = find_linked_list_end(t, b);
    if (t->excess_size == 0)
        return 0;
    int64_t p = t->excess[--t->excess_size]; /* vector::pop_back: vector_detail.cuh:240-299 */
    t->keys[p] = key;
    t->vals[p] = value;
    t->hashes[p] = hash;
    t->offsets[p] = 0;
    ++t->occupied_count;
    t->occupied[p] = 1;
    t->offsets[end] = p - end;
    return 1;
}

int port_insert(port_table* t, uint64_t key, uint64_t value)
{
    return port_insert_h(t, key, key, value);
}

/* erase(key) retry loop :1019-1043 around try_erase :811-913, run by one thread */
int port_erase_h(port_table* t, uint64_t key, uint64_t hash)
{
    int64_t p = find_pos_h(t, key, hash);
    if (p < 0)
        return 0;
    int64_t b = port_fibonacci_hashing(hash, t->bucket_count);
    if (p == b)
    {
        /* :826-857 bucket head: reset occupancy, leave the chain link */
        t->occupied[p] = 0;
        --t->occupied_count;
        return 1;
    }
    /* :858-905 chain entry: unlink, reset occupancy, return the slot to the excess list */
    int64_t prev = find_previous_entry_position(t, p, b);
    if (t->offsets[p] != 0)
        t->offsets[prev] += t->offsets[p];
    else
        t->offsets[prev] = 0;
    t->occupied[p] = 0;
    --t->occupied_count;
    t->excess[t->excess_size++] = p; /* vector::push_back: vector_detail.cuh:181-238 */
    return 1;
}

int port_erase(port_table* t, uint64_t key)
{
    return port_erase_h(t, key, key);
}

/* bulk forms with caller-supplied hashes (a user Hash functor); flags / values / found may be NULL */
void port_insert_bulk_h(port_table* t, const uint64_t* keys, const uint64_t* hashes, const uint64_t* values, int64_t n,
                        uint8_t* flags)
{
    for (int64_t i = 0; i < n; ++i)
    {
        int r = port_insert_h(t, keys[i], hashes[i], values ? values[i] : 0);
        if (flags)
            flags[i] = (uint8_t)r;
    }
}

void port_erase_bulk_h(port_table* t, const uint64_t* keys, const uint64_t* hashes, int64_t n, uint8_t* flags)
{
    for (int64_t i = 0; i < n; ++i)
    {
        int r = port_erase_h(t, keys[i], hashes[i]);
        if (flags)
            flags[i] = (uint8_t)r;
    }
}

void port_find_bulk_h(const port_table* t, const uint64_t* keys, const uint64_t* hashes, int64_t n, uint64_t* values,
                      uint8_t* found)
{
    for (int64_t i = 0; i < n; ++i)
    {
        uint64_t v = 0;
        int r = port_find_h(t, keys[i], hashes[i], &v);
        if (found)
            found[i] = (uint8_t)r;
        if (values)
            values[i] = r ? v : 0;
    }
}

/* bulk insert(begin,end): :996-1017 -- one insert(value) per element */
void port_insert_bulk(port_table* t, const uint64_t* keys, const uint64_t* values, int64_t n, uint8_t* flags)
{
    for (int64_t i = 0; i < n; ++i)
    {
        int r = port_insert(t, keys[i], values ? values[i] : 0);
        if (flags)
            flags[i] = (uint8_t)r;
    }
}

/* bulk erase(begin,end): :1045-1066 -- one erase(key) per element */
void port_erase_bulk(port_table* t, const uint64_t* keys, int64_t n, uint8_t* flags)
{
    for (int64_t i = 0; i < n; ++i)
    {
        int r = port_erase(t, keys[i]);
        if (flags)
            flags[i] = (uint8_t)r;
    }
}

void port_find_bulk(const port_table* t, const uint64_t* keys, int64_t n, uint64_t* values, uint8_t* found)
{
    for (int64_t i = 0; i < n; ++i)
    {
        uint64_t v = 0;
        int r = port_find(t, keys[i], &v);
        if (found)
            found[i] = (uint8_t)r;
        if (values)
            values[i] = r ? v : 0;
    }
}

/* size / bucket_count / max_size: :1110-1153 */
int64_t port_size(const port_table* t) { return t->occupied_count; }
int64_t port_bucket_count(const port_table* t) { return t->bucket_count; }
int64_t port_max_size(const port_table* t) { return t->total_count; }
/* slots taken from the excess list: excess_count minus _excess_list_positions.size() */
int64_t port_excess_used(const port_table* t) { return t->excess_count - t->excess_size; }

/* bucket_size(n): :566-593 */
int64_t port_bucket_size(const port_table* t, int64_t n)
{
    int64_t r = 0;
    int64_t i = n;
    if (t->occupied[i])
        ++r;
    while (t->offsets[i] != 0)
    {
        i += t->offsets[i];
        if (t->occupied[i])
            ++r;
    }
    return r;
}

/* clear(): :1220-1252 (returns early on an empty table, leaving links and the free-list as they are) */
void port_clear(port_table* t)
{
    if (t->occupied_count == 0)
        return;
    memset(t->offsets, 0, (size_t)t->total_count * sizeof(int64_t));
    memset(t->occupied, 0, (size_t)t->total_count);
    t->occupied_count = 0;
    reset_excess(t);
}

/* valid(): :1192-1218 with the checkers of :210-468 */
int port_valid(const port_table* t)
{
    if (t->total_count == 0)
        return 1;
    /* offset_inside_range :210-256 */
    for (int64_t i = 0; i < t->total_count; ++i)
    {
        int64_t l = i + t->offsets[i];
        if (l < 0 || l >= t->total_count)
            return 0;
    }
    /* loop_free :258-350 -- chains from distinct buckets visit every slot at most once */
    int* flags = (int*)calloc((size_t)t->total_count, sizeof(int));
    int ok = 1;
    for (int64_t b = 0; b < t->bucket_count && ok; ++b)
    {
        int64_t i = b;
        ++flags[i];
        while (t->offsets[i] != 0)
        {
            i += t->offsets[i];
            ++flags[i];
            if (flags[i] > 1)
            {
                ok = 0;
                break;
            }
        }
    }
    for (int64_t i = 0; i < t->total_count && ok; ++i)
        if (flags[i] > 1)
            ok = 0;
    free(flags);
    if (!ok)
        return 0;
    /* values_reachable :352-398 and unique :400-451 */
    int64_t pop = 0;
    for (int64_t i = 0; i < t->total_count; ++i)
    {
        if (!t->occupied[i])
            continue;
        ++pop;
        if (find_pos_h(t, t->keys[i], t->hashes[i]) != i)
            return 0;
    }
    /* occupied_count_valid :453-468 */
    return pop == t->occupied_count;
}

/* device_range(): :160-208 (the reference collects in a nondeterministic order; here slot order) */
int64_t port_range(const port_table* t, uint64_t* keys, uint64_t* values)
{
    int64_t n = 0;
    for (int64_t i = 0; i < t->total_count; ++i)
    {
        if (!t->occupied[i])
            continue;
        if (keys)
            keys[n] = t->keys[i];
        if (values)
            values[n] = t->vals[i];
        ++n;
    }
    return n;
}

/* vector<T>::push_back run by one thread per element in index order: src/stdgpu/impl/vector_detail.cuh:181-238;
 * size() clamps to capacity (:484-511) */
int64_t port_vector_push_back(int64_t capacity, const uint64_t* values, const uint8_t* pred, int64_t n,
                              uint8_t* pushed, uint64_t* out)
{
    int64_t size = 0;
    for (int64_t i = 0; i < n; ++i)
    {
        uint8_t ok = 0;
        if (!pred || pred[i])
        {
            int64_t clamped = size > capacity ? capacity : size;
            if (clamped != capacity) /* :187-192 preemptive full() check */
            {
                int64_t pos = size++;
                if (pos < capacity)
                {
                    if (out)
                        out[pos] = values[i];
                    ok = 1;
                }
            }
        }
        if (pushed)
            pushed[i] = ok;
    }
    return size > capacity ? capacity : size;
}

/* deque<T> push_back :202-258 and pop_front :388-446 of src/stdgpu/impl/deque_detail.cuh, sequentially;
 * positions advance with fetch_inc_mod(capacity) (src/stdgpu/impl/atomic_detail.cuh:675-687) */
int64_t port_deque_ops(int64_t capacity, const uint64_t* init, int64_t n_init, const uint8_t* is_push,
                       const uint64_t* values, int64_t n, uint64_t* popped, uint8_t* ok, uint64_t* remaining)
{
    uint64_t* data = (uint64_t*)calloc((size_t)(capacity > 0 ? capacity : 1), sizeof(uint64_t));
    int64_t size = 0, begin = 0, end = 0;
    for (int64_t j = 0; j < n_init + n; ++j)
    {
        /* op: 0 pop_front, 1 push_back, 2 push_front (:314-386), 3 pop_back (:260-312) */
        int op = j < n_init ? 1 : is_push[j - n_init];
        int push = op == 1 || op == 2;
        uint64_t v = j < n_init ? init[j] : values[j - n_init];
        uint8_t r = 0;
        uint64_t pv = 0;
        if (op == 2)
        {
            if (size != capacity)
            {
                int64_t cur = size++;
                if (cur < capacity)
                {
                    /* begin.fetch_dec_mod(capacity), then the position before the old begin */
                    begin = (begin == 0) ? capacity - 1 : begin - 1;
                    data[begin] = v;
                    r = 1;
                }
            }
        }
        else if (op == 3)
        {
            if (size != 0)
            {
                int64_t cur = size--;
                if (cur > 0)
                {
                    end = (end == 0) ? capacity - 1 : end - 1;
                    pv = data[end];
                    r = 1;
                }
            }
        }
        else if (push)
        {
            if (size != capacity)
            {
                int64_t cur = size++;
                if (cur < capacity)
                {
                    int64_t pos = end;
                    end = (end >= capacity - 1) ? 0 : end + 1;
                    data[pos] = v;
                    r = 1;
                }
            }
        }
        else
        {
            if (size != 0)
            {
                int64_t cur = size--;
                if (cur > 0)
                {
                    int64_t pos = begin;
                    begin = (begin >= capacity - 1) ? 0 : begin + 1;
                    pv = data[pos];
                    r = 1;
                }
            }
        }
        if (j >= n_init)
        {
            if (ok)
                ok[j - n_init] = r;
            if (popped && !push)
                popped[j - n_init] = pv;
        }
    }
    if (remaining)
        for (int64_t i = 0; i < size; ++i)
            remaining[i] = data[(begin + i) % capacity];
    free(data);
    return size;
}

/* count_block_bits + bitset::count: src/stdgpu/impl/bitset_detail.cuh:130-160, 388-404 */
int64_t port_bitset_count(const uint32_t* words, int64_t nbits)
{
    if (nbits == 0)
        return 0;
    int64_t blocks = (nbits + 31) / 32;
    int64_t c = 0;
    for (int64_t i = 0; i < blocks; ++i)
    {
        int64_t remaining = nbits - i * 32;
        uint32_t mask = remaining >= 32 ? 0xFFFFFFFFu : ((1u << remaining) - 1u);
        c += __builtin_popcount(words[i] & mask);
    }
    return c;
}

// Test infrastructure only: a C entry layer over the reference library itself
// (stdgpu 1.3.0, OpenMP backend), used as the checker for the CUDA path and as
// the reference CPU baseline.  It is never linked into the product library.
//
// Every entry point drives the reference through its own public API:
//   createDeviceObject / destroyDeviceObject  src/stdgpu/impl/unordered_base_detail.cuh:1254-1348
//   bulk insert(begin,end)                    src/stdgpu/impl/unordered_base_detail.cuh:996-1017
//   bulk erase(begin,end)                     src/stdgpu/impl/unordered_base_detail.cuh:1045-1066
//   device find / contains / insert / erase   src/stdgpu/impl/unordered_base_detail.cuh:619-706, 958-994, 1019-1043
//   size / valid / clear / device_range       src/stdgpu/impl/unordered_base_detail.cuh:1110-1252, 160-208
//   vector::push_back                         src/stdgpu/impl/vector_detail.cuh:181-238
//   deque::push_back / pop_front              src/stdgpu/impl/deque_detail.cuh:202-258, 388-446
//   bitset::set / count                       src/stdgpu/impl/bitset_detail.cuh:46-112, 388-404
// Under the OpenMP backend "device" memory is host memory, so host arrays are
// passed straight through `stdgpu::make_device`.

#include <cstdint>
#include <cstdlib>
#include <chrono>
#include <cstring>
#include <new>
#include <unordered_map>
#include <vector>

#include <stdgpu/algorithm.h>
#include <stdgpu/bitset.cuh>
#include <stdgpu/deque.cuh>
#include <stdgpu/iterator.h>
#include <stdgpu/memory.h>
#include <stdgpu/unordered_map.cuh>
#include <stdgpu/unordered_set.cuh>
#include <stdgpu/vector.cuh>

#include <omp.h>

namespace
{

enum kind_t
{
    SET_U32 = 0,
    SET_U64 = 1,
    MAP_U64_U32 = 2,
    MAP_U64_U64 = 3,
    MAP_U32_U32 = 4,
    MAP_U32_U64 = 5,
    SET_VEC3I16 = 6,     // unordered_set<vec3i16, spatial_hash>
    MAP_VEC3I16_U32 = 7, // unordered_map<vec3i16, uint32_t, spatial_hash>
    SET_VEC3I32 = 8,     // unordered_set<vec3i32, spatial_hash>
    MAP_VEC3I32_U64 = 9, // unordered_map<vec3i32, uint64_t, spatial_hash>
};

// A custom key type and hash as the reference's users write them (the reference's own tests use a
// 3 x int16 key with this hash: tests/stdgpu/unordered_map.inc:178-206).  The hash is the spatial hash
// of Teschner et al., "Optimized Spatial Hashing for Collision Detection of Deformable Objects" (2003):
// each coordinate, sign-extended to 64 bits, times one of three large primes, combined by xor.
struct vec3i16
{
    std::int16_t x = 0;
    std::int16_t y = 0;
    std::int16_t z = 0;
};

inline bool
operator==(const vec3i16& a, const vec3i16& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}

// A 12-byte key with a user-declared destructor, the shape of the reference's nontrivial-type tests
// (tests/stdgpu/unordered_map.inc:132-161).
struct vec3i32
{
    vec3i32() = default;
    vec3i32(const vec3i32&) = default;
    vec3i32& operator=(const vec3i32&) = default;
    ~vec3i32() {}

    std::int32_t x = 0;
    std::int32_t y = 0;
    std::int32_t z = 0;
};

inline bool
operator==(const vec3i32& a, const vec3i32& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}

struct spatial_hash
{
    std::size_t
    operator()(const vec3i16& k) const
    {
        return (static_cast<std::size_t>(k.x) * static_cast<std::size_t>(73856093U)) ^
               (static_cast<std::size_t>(k.y) * static_cast<std::size_t>(19349669U)) ^
               (static_cast<std::size_t>(k.z) * static_cast<std::size_t>(83492791U));
    }
    std::size_t
    operator()(const vec3i32& k) const
    {
        return (static_cast<std::size_t>(k.x) * static_cast<std::size_t>(73856093U)) ^
               (static_cast<std::size_t>(k.y) * static_cast<std::size_t>(19349669U)) ^
               (static_cast<std::size_t>(k.z) * static_cast<std::size_t>(83492791U));
    }
};

struct table_base
{
    virtual ~table_base() = default;
    virtual void insert(const void* keys, const void* vals, std::int64_t n) = 0;
    virtual void insert_flags(const void* keys, const void* vals, std::int64_t n, std::uint8_t* flags) = 0;
    virtual void erase(const void* keys, std::int64_t n) = 0;
    virtual void erase_flags(const void* keys, std::int64_t n, std::uint8_t* flags) = 0;
    virtual void find(const void* keys, std::int64_t n, void* out_vals, std::uint8_t* found) = 0;
    virtual void contains(const void* keys, std::int64_t n, std::uint8_t* flags) = 0;
    virtual std::int64_t size() = 0;
    virtual int valid() = 0;
    virtual void clear() = 0;
    virtual std::int64_t range(void* out_keys, void* out_vals) = 0;
    virtual std::int64_t bucket(const void* key) = 0;
    virtual void geometry(std::int64_t* bucket_count, std::int64_t* max_size) = 0;
};

// ---- key/value plumbing: sets carry Key, maps carry pair<const Key, T> ----

template <typename Key, typename Hash = stdgpu::hash<Key>>
struct set_traits
{
    using container = stdgpu::unordered_set<Key, Hash>;
    using key_type = Key;
    using mapped_type = std::uint8_t; // unused
    using value_type = Key;
    static constexpr bool is_map = false;

    static value_type
    make(const Key& k, const mapped_type& /*v*/)
    {
        return k;
    }
    static const Key&
    key_of(const value_type& v)
    {
        return v;
    }
};

template <typename Key, typename T, typename Hash = stdgpu::hash<Key>>
struct map_traits
{
    using container = stdgpu::unordered_map<Key, T, Hash>;
    using key_type = Key;
    using mapped_type = T;
    using value_type = stdgpu::pair<const Key, T>;
    static constexpr bool is_map = true;

    static value_type
    make(const Key& k, const T& v)
    {
        return value_type(k, v);
    }
    static const Key&
    key_of(const value_type& v)
    {
        return v.first;
    }
};

template <typename Traits>
struct insert_flag_functor
{
    typename Traits::container c;
    const typename Traits::value_type* values;
    std::uint8_t* flags;

    void
    operator()(const stdgpu::index_t i)
    {
        flags[i] = c.insert(values[i]).second ? 1 : 0;
    }
};

template <typename Traits>
struct erase_flag_functor
{
    typename Traits::container c;
    const typename Traits::key_type* keys;
    std::uint8_t* flags;

    void
    operator()(const stdgpu::index_t i)
    {
        flags[i] = static_cast<std::uint8_t>(c.erase(keys[i]));
    }
};

template <typename Traits>
struct find_functor
{
    typename Traits::container c;
    const typename Traits::key_type* keys;
    typename Traits::mapped_type* out;
    std::uint8_t* found;

    void
    operator()(const stdgpu::index_t i)
    {
        auto it = c.find(keys[i]);
        if (it != c.end())
        {
            found[i] = 1;
            if constexpr (Traits::is_map)
            {
                if (out != nullptr)
                {
                    out[i] = it->second;
                }
            }
        }
        else
        {
            found[i] = 0;
        }
    }
};

template <typename Traits>
struct contains_functor
{
    typename Traits::container c;
    const typename Traits::key_type* keys;
    std::uint8_t* flags;

    void
    operator()(const stdgpu::index_t i)
    {
        flags[i] = c.contains(keys[i]) ? 1 : 0;
    }
};

template <typename Traits>
struct table_impl final : table_base
{
    using K = typename Traits::key_type;
    using V = typename Traits::mapped_type;
    using VT = typename Traits::value_type;

    typename Traits::container c;

    explicit table_impl(std::int64_t capacity)
      : c(Traits::container::createDeviceObject(static_cast<stdgpu::index_t>(capacity)))
    {
    }

    ~table_impl() override { Traits::container::destroyDeviceObject(c); }

    // value_type holds a const key, so build the array in raw storage
    static VT*
    build_values(const void* keys, const void* vals, std::int64_t n)
    {
        auto* raw = static_cast<VT*>(std::malloc(sizeof(VT) * static_cast<std::size_t>(n > 0 ? n : 1)));
        const K* k = static_cast<const K*>(keys);
        const V* v = static_cast<const V*>(vals);
        for (std::int64_t i = 0; i < n; ++i)
        {
            V vi = (Traits::is_map && v != nullptr) ? v[i] : V{};
            new (raw + i) VT(Traits::make(k[i], vi));
        }
        return raw;
    }

    void
    insert(const void* keys, const void* vals, std::int64_t n) override
    {
        VT* values = build_values(keys, vals, n);
        c.insert(stdgpu::make_device(static_cast<const VT*>(values)),
                 stdgpu::make_device(static_cast<const VT*>(values + n)));
        std::free(values);
    }

    void
    insert_flags(const void* keys, const void* vals, std::int64_t n, std::uint8_t* flags) override
    {
        VT* values = build_values(keys, vals, n);
        stdgpu::for_each_index(stdgpu::execution::device,
                               static_cast<stdgpu::index_t>(n),
                               insert_flag_functor<Traits>{ c, values, flags });
        std::free(values);
    }

    void
    erase(const void* keys, std::int64_t n) override
    {
        const K* k = static_cast<const K*>(keys);
        c.erase(stdgpu::make_device(k), stdgpu::make_device(k + n));
    }

    void
    erase_flags(const void* keys, std::int64_t n, std::uint8_t* flags) override
    {
        stdgpu::for_each_index(stdgpu::execution::device,
                               static_cast<stdgpu::index_t>(n),
                               erase_flag_functor<Traits>{ c, static_cast<const K*>(keys), flags });
    }

    void
    find(const void* keys, std::int64_t n, void* out_vals, std::uint8_t* found) override
    {
        stdgpu::for_each_index(stdgpu::execution::device,
                               static_cast<stdgpu::index_t>(n),
                               find_functor<Traits>{ c, static_cast<const K*>(keys), static_cast<V*>(out_vals), found });
    }

    void
    contains(const void* keys, std::int64_t n, std::uint8_t* flags) override
    {
        stdgpu::for_each_index(stdgpu::execution::device,
                               static_cast<stdgpu::index_t>(n),
                               contains_functor<Traits>{ c, static_cast<const K*>(keys), flags });
    }

    std::int64_t
    size() override
    {
        return static_cast<std::int64_t>(c.size());
    }

    int
    valid() override
    {
        return c.valid() ? 1 : 0;
    }

    void
    clear() override
    {
        c.clear();
    }

    std::int64_t
    range(void* out_keys, void* out_vals) override
    {
        auto r = c.device_range();
        std::int64_t n = 0;
        K* ok = static_cast<K*>(out_keys);
        V* ov = static_cast<V*>(out_vals);
        for (auto it = r.begin(); it != r.end(); ++it, ++n)
        {
            const VT& v = *it;
            if (ok != nullptr)
            {
                ok[n] = Traits::key_of(v);
            }
            if constexpr (Traits::is_map)
            {
                if (ov != nullptr)
                {
                    ov[n] = v.second;
                }
            }
        }
        return n;
    }

    std::int64_t
    bucket(const void* key) override
    {
        return static_cast<std::int64_t>(c.bucket(*static_cast<const K*>(key)));
    }

    void
    geometry(std::int64_t* bucket_count, std::int64_t* max_size) override
    {
        *bucket_count = static_cast<std::int64_t>(c.bucket_count());
        *max_size = static_cast<std::int64_t>(c.max_size());
    }
};

// ---- vector, deque and bitset entry points ----

struct vec_push_functor
{
    stdgpu::vector<std::uint32_t> v;
    const std::uint32_t* values;
    const std::uint8_t* pred;
    std::uint8_t* pushed;

    void
    operator()(const stdgpu::index_t i)
    {
        std::uint8_t ok = 0;
        if (pred == nullptr || pred[i] != 0)
        {
            ok = v.push_back(values[i]) ? 1 : 0;
        }
        if (pushed != nullptr)
        {
            pushed[i] = ok;
        }
    }
};

struct deque_op_functor
{
    stdgpu::deque<std::uint64_t> d;
    const std::uint8_t* is_push;
    const std::uint64_t* values;
    std::uint64_t* popped;
    std::uint8_t* ok;

    // is_push[i]: 0 pop_front, 1 push_back, 2 push_front, 3 pop_back
    void
    operator()(const stdgpu::index_t i)
    {
        if (is_push[i] == 1 || is_push[i] == 2)
        {
            ok[i] = (is_push[i] == 1 ? d.push_back(values[i]) : d.push_front(values[i])) ? 1 : 0;
        }
        else
        {
            stdgpu::pair<std::uint64_t, bool> r = is_push[i] == 0 ? d.pop_front() : d.pop_back();
            ok[i] = r.second ? 1 : 0;
            popped[i] = r.second ? r.first : 0;
        }
    }
};

struct bitset_load_functor
{
    stdgpu::bitset<> b;
    const std::uint32_t* words;

    void
    operator()(const stdgpu::index_t i)
    {
        if ((words[i / 32] >> (i % 32)) & 1U)
        {
            b.set(i);
        }
    }
};

} // namespace

extern "C" {

int
sgref_index_bits(void)
{
    return static_cast<int>(sizeof(stdgpu::index_t) * 8);
}

void
sgref_set_threads(int n)
{
    omp_set_num_threads(n);
}

int
sgref_max_threads(void)
{
    return omp_get_max_threads();
}

void*
sgref_create(int kind, std::int64_t capacity)
{
    switch (kind)
    {
        case SET_U32:
            return new table_impl<set_traits<std::uint32_t>>(capacity);
        case SET_U64:
            return new table_impl<set_traits<std::uint64_t>>(capacity);
        case MAP_U64_U32:
            return new table_impl<map_traits<std::uint64_t, std::uint32_t>>(capacity);
        case MAP_U64_U64:
            return new table_impl<map_traits<std::uint64_t, std::uint64_t>>(capacity);
        case MAP_U32_U32:
            return new table_impl<map_traits<std::uint32_t, std::uint32_t>>(capacity);
        case MAP_U32_U64:
            return new table_impl<map_traits<std::uint32_t, std::uint64_t>>(capacity);
        case SET_VEC3I16:
            return new table_impl<set_traits<vec3i16, spatial_hash>>(capacity);
        case MAP_VEC3I16_U32:
            return new table_impl<map_traits<vec3i16, std::uint32_t, spatial_hash>>(capacity);
        case SET_VEC3I32:
            return new table_impl<set_traits<vec3i32, spatial_hash>>(capacity);
        case MAP_VEC3I32_U64:
            return new table_impl<map_traits<vec3i32, std::uint64_t, spatial_hash>>(capacity);
        default:
            return nullptr;
    }
}

void
sgref_destroy(void* h)
{
    delete static_cast<table_base*>(h);
}

void
sgref_insert(void* h, const void* keys, const void* vals, std::int64_t n)
{
    static_cast<table_base*>(h)->insert(keys, vals, n);
}

void
sgref_insert_flags(void* h, const void* keys, const void* vals, std::int64_t n, std::uint8_t* flags)
{
    static_cast<table_base*>(h)->insert_flags(keys, vals, n, flags);
}

void
sgref_erase(void* h, const void* keys, std::int64_t n)
{
    static_cast<table_base*>(h)->erase(keys, n);
}

void
sgref_erase_flags(void* h, const void* keys, std::int64_t n, std::uint8_t* flags)
{
    static_cast<table_base*>(h)->erase_flags(keys, n, flags);
}

void
sgref_find(void* h, const void* keys, std::int64_t n, void* out_vals, std::uint8_t* found)
{
    static_cast<table_base*>(h)->find(keys, n, out_vals, found);
}

void
sgref_contains(void* h, const void* keys, std::int64_t n, std::uint8_t* flags)
{
    static_cast<table_base*>(h)->contains(keys, n, flags);
}

std::int64_t
sgref_size(void* h)
{
    return static_cast<table_base*>(h)->size();
}

int
sgref_valid(void* h)
{
    return static_cast<table_base*>(h)->valid();
}

void
sgref_clear(void* h)
{
    static_cast<table_base*>(h)->clear();
}

std::int64_t
sgref_range(void* h, void* out_keys, void* out_vals)
{
    return static_cast<table_base*>(h)->range(out_keys, out_vals);
}

std::int64_t
sgref_bucket(void* h, const void* key)
{
    return static_cast<table_base*>(h)->bucket(key);
}

void
sgref_geometry(void* h, std::int64_t* bucket_count, std::int64_t* max_size)
{
    static_cast<table_base*>(h)->geometry(bucket_count, max_size);
}

// vector<uint32_t>: thread i pushes values[i] when pred[i] != 0 (pred may be NULL);
// returns size() afterwards and writes the contents (in storage order) to out.
std::int64_t
sgref_vector_push_back(std::int64_t capacity,
                       const std::uint32_t* values,
                       const std::uint8_t* pred,
                       std::int64_t n,
                       std::uint8_t* pushed,
                       std::uint32_t* out)
{
    auto v = stdgpu::vector<std::uint32_t>::createDeviceObject(static_cast<stdgpu::index_t>(capacity));
    stdgpu::for_each_index(stdgpu::execution::device,
                           static_cast<stdgpu::index_t>(n),
                           vec_push_functor{ v, values, pred, pushed });
    std::int64_t size = static_cast<std::int64_t>(v.size());
    if (out != nullptr)
    {
        std::memcpy(out, v.data(), static_cast<std::size_t>(size) * sizeof(std::uint32_t));
    }
    stdgpu::vector<std::uint32_t>::destroyDeviceObject(v);
    return size;
}

// deque<uint64_t>: `n_init` sequential push_backs, then one parallel launch of
// mixed ops (is_push[i] ? push_back(values[i]) : pop_front()).  Returns size()
// afterwards; the remaining elements are written front-to-back to `remaining`.
std::int64_t
sgref_deque_ops(std::int64_t capacity,
                const std::uint64_t* init,
                std::int64_t n_init,
                const std::uint8_t* is_push,
                const std::uint64_t* values,
                std::int64_t n,
                std::uint64_t* popped,
                std::uint8_t* ok,
                std::uint64_t* remaining)
{
    auto d = stdgpu::deque<std::uint64_t>::createDeviceObject(static_cast<stdgpu::index_t>(capacity));
    std::vector<std::uint8_t> init_push(static_cast<std::size_t>(n_init > 0 ? n_init : 1), 1);
    std::vector<std::uint64_t> init_pop(static_cast<std::size_t>(n_init > 0 ? n_init : 1), 0);
    std::vector<std::uint8_t> init_ok(static_cast<std::size_t>(n_init > 0 ? n_init : 1), 0);
    if (n_init > 0)
    {
        stdgpu::for_each_index(stdgpu::execution::device,
                               static_cast<stdgpu::index_t>(n_init),
                               deque_op_functor{ d, init_push.data(), init, init_pop.data(), init_ok.data() });
    }
    if (n > 0)
    {
        stdgpu::for_each_index(stdgpu::execution::device,
                               static_cast<stdgpu::index_t>(n),
                               deque_op_functor{ d, is_push, values, popped, ok });
    }
    std::int64_t size = static_cast<std::int64_t>(d.size());
    if (remaining != nullptr)
    {
        for (std::int64_t i = 0; i < size; ++i)
        {
            remaining[i] = d.at(static_cast<stdgpu::index_t>(i));
        }
    }
    stdgpu::deque<std::uint64_t>::destroyDeviceObject(d);
    return size;
}

// bitset of `nbits` bits whose bit i is bit (i % 32) of words[i / 32]; returns count().
std::int64_t
sgref_bitset_count(const std::uint32_t* words, std::int64_t nbits)
{
    auto b = stdgpu::bitset<>::createDeviceObject(static_cast<stdgpu::index_t>(nbits));
    stdgpu::for_each_index(stdgpu::execution::device,
                           static_cast<stdgpu::index_t>(nbits),
                           bitset_load_functor{ b, words });
    std::int64_t c = static_cast<std::int64_t>(b.count());
    stdgpu::bitset<>::destroyDeviceObject(b);
    return c;
}

// Sanity line beside the reference: the same insert / find / erase sequence on std::unordered_map<uint64_t,
// uint32_t> in one thread (reserved for n elements).  Returns the wall seconds of the three phases; hits,
// value_sum (of the values found) and final_size report what it did, so no part of the work can be dropped.
double
sgref_std_unordered_map_run(const std::uint64_t* keys, const std::uint32_t* vals, std::int64_t n,
                            const std::uint64_t* queries, std::int64_t nq, const std::uint64_t* erase,
                            std::int64_t ne, std::int64_t* hits, std::uint64_t* value_sum, std::int64_t* final_size)
{
    std::unordered_map<std::uint64_t, std::uint32_t> m;
    m.reserve(static_cast<std::size_t>(n));
    const auto t0 = std::chrono::steady_clock::now();
    for (std::int64_t i = 0; i < n; ++i)
    {
        m.emplace(keys[i], vals[i]);
    }
    std::int64_t h = 0;
    std::uint64_t sum = 0;
    for (std::int64_t i = 0; i < nq; ++i)
    {
        const auto it = m.find(queries[i]);
        if (it != m.end())
        {
            ++h;
            sum += it->second;
        }
    }
    for (std::int64_t i = 0; i < ne; ++i)
    {
        m.erase(erase[i]);
    }
    const auto t1 = std::chrono::steady_clock::now();
    *hits = h;
    *value_sum = sum;
    *final_size = static_cast<std::int64_t>(m.size());
    return std::chrono::duration<double>(t1 - t0).count();
}

} // extern "C"

// C++ host API with the reference's names over the C ABI of this library.
//
// A translation unit that used stdgpu's hashed containers
// (src/stdgpu/unordered_map.cuh, src/stdgpu/unordered_set.cuh, src/stdgpu/vector.cuh,
// src/stdgpu/deque.cuh, src/stdgpu/bitset.cuh) for 4/8-byte integer keys includes this header
// instead and keeps its calls: createDeviceObject / destroyDeviceObject, bulk insert(begin, end) /
// erase(begin, end), size / empty / full / max_size / bucket_count / load_factor / clear / valid /
// device_range, and inside its own kernels the device members find / contains / count / insert /
// emplace / erase / bucket / bucket_size.  Objects are shallow handles copied by value into kernels,
// as in the reference (docs/api/object.md); exactly one destroyDeviceObject frees them.
//
// Errors: like the reference (src/stdgpu/cuda/impl/error.h:41-56), a failed call prints and
// terminates by default; set stdgpu::gb300_error_handler to change that.
#ifndef STDGPU_GB300_STDGPU_CUH
#define STDGPU_GB300_STDGPU_CUH

#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <exception>
#include <functional>
#include <memory>
#include <mutex>
#include <type_traits>
#include <unordered_map>

#include "../stdgpu_gb300.h"
#include "device.cuh"

namespace stdgpu
{

using index_t = std::int32_t; // the reference's default index type (src/stdgpu/cstddef.h:42-59)

// stdgpu::hash: the identity for integer keys (src/stdgpu/impl/functional_detail.h:60-80).  Other key types
// bring their own Hash.
template <typename Key>
struct hash
{
    template <typename K = Key, typename = std::enable_if_t<std::is_integral<K>::value>>
    __host__ __device__ std::size_t
    operator()(const Key& key) const
    {
        return static_cast<std::size_t>(key);
    }
};

// stdgpu::equal_to (src/stdgpu/functional.h); equal_to<void> compares any two comparable values.
template <typename T = void>
struct equal_to
{
    __host__ __device__ bool
    operator()(const T& a, const T& b) const
    {
        return a == b;
    }
};
template <>
struct equal_to<void>
{
    using is_transparent = void;
    template <typename A, typename B>
    __host__ __device__ bool
    operator()(const A& a, const B& b) const
    {
        return a == b;
    }
};

inline void (*gb300_error_handler)(sg_status, const char*) = [](sg_status st, const char* what) {
    std::fprintf(stderr, "stdgpu_gb300: %s failed: %s\n", what, sg_status_string(st));
    std::terminate();
};

namespace detail
{
inline void
gb300_check(sg_status st, const char* what)
{
    if (st != SG_OK)
    {
        gb300_error_handler(st, what);
    }
}
} // namespace detail

// stdgpu::pair (src/stdgpu/utility.h); pair<const Key, T> has the reference's byte layout.
template <typename T1, typename T2>
struct pair
{
    T1 first;
    T2 second;

    pair() = default;
    __host__ __device__ constexpr pair(const T1& a, const T2& b)
      : first(a)
      , second(b)
    {
    }
};

// stdgpu::safe_device_allocator<T> (src/stdgpu/memory.h:340-420): device memory through cudaMalloc / cudaFree.
// The containers take an allocator type parameter, as the reference's do.  With this default type a
// container's storage goes through the library's allocator pair (sg_set_device_allocator, one per process);
// an unordered_map / unordered_set created with another allocator (createDeviceObject(capacity, allocator))
// takes all of its device storage from that allocator (detail::allocator_bridge), and get_allocator()
// returns it.
template <typename T>
struct safe_device_allocator
{
    using value_type = T;

    safe_device_allocator() noexcept = default;

    template <typename U>
    safe_device_allocator(const safe_device_allocator<U>&) noexcept
    {
    }

    T*
    allocate(std::int64_t n)
    {
        T* p = nullptr;
        detail::gb300_check(cudaMalloc(&p, sizeof(T) * static_cast<std::size_t>(n)) == cudaSuccess ? SG_OK : SG_ERR_OOM,
                            "safe_device_allocator::allocate");
        return p;
    }

    void
    deallocate(T* p, std::int64_t)
    {
        cudaFree(p);
    }
};

namespace detail
{
template <typename Allocator>
struct is_safe_device_allocator : std::false_type
{
};
template <typename T>
struct is_safe_device_allocator<safe_device_allocator<T>> : std::true_type
{
};

// The sg_allocator of a C++ Allocator: byte blocks through std::allocator_traits of the allocator rebound to
// char, as the reference allocates its arrays (src/stdgpu/impl/memory_detail.h, allocator_traits); the
// context owns a copy of the allocator and the size of every block it handed out (deallocate takes it) and
// is deleted with the table (release_ctx).
template <typename Allocator>
struct allocator_bridge
{
    using bytes = typename std::allocator_traits<Allocator>::template rebind_alloc<char>;
    using traits = std::allocator_traits<bytes>;

    bytes a;
    std::mutex m;
    std::unordered_map<void*, std::size_t> sizes;

    explicit allocator_bridge(const Allocator& x)
      : a(x)
    {
    }

    static void*
    alloc(std::size_t n, void* c)
    {
        auto* x = static_cast<allocator_bridge*>(c);
        char* p = traits::allocate(x->a, static_cast<typename traits::size_type>(n));
        if (p != nullptr)
        {
            std::lock_guard<std::mutex> lock(x->m);
            x->sizes[p] = n;
        }
        return p;
    }

    static void
    release(void* p, void* c)
    {
        auto* x = static_cast<allocator_bridge*>(c);
        std::size_t n = 0;
        {
            std::lock_guard<std::mutex> lock(x->m);
            auto it = x->sizes.find(p);
            if (it == x->sizes.end())
            {
                return;
            }
            n = it->second;
            x->sizes.erase(it);
        }
        traits::deallocate(x->a, static_cast<char*>(p), static_cast<typename traits::size_type>(n));
    }

    static void
    drop(void* c)
    {
        delete static_cast<allocator_bridge*>(c);
    }

    static sg_allocator
    make(const Allocator& x)
    {
        return sg_allocator{ &alloc, &release, new allocator_bridge(x), &drop };
    }
};

// A block of an object's own allocator (nullptr when its alloc is empty or fails).
template <typename P>
inline P*
own_alloc(const sg_allocator& a, std::size_t bytes)
{
    return a.alloc != nullptr ? static_cast<P*>(a.alloc(bytes > 0 ? bytes : 1, a.ctx)) : nullptr;
}
} // namespace detail

// Execution policies: the reference's execution::device plus a stream-carrying policy.
namespace execution
{
struct device_policy
{
    cudaStream_t stream = nullptr;
};
inline constexpr device_policy device{};
inline device_policy
on(cudaStream_t s)
{
    return device_policy{ s };
}
} // namespace execution

// Result of device_range(): stored elements addressed through slot indices, in slot order.
template <typename T>
struct device_indexed_range
{
    const std::int32_t* indices = nullptr;
    index_t count = 0;
    T* values = nullptr;

    __host__ __device__ index_t
    size() const
    {
        return count;
    }
    __device__ T&
    operator[](index_t i) const
    {
        return values[indices[i]];
    }
};

namespace detail
{
template <typename Key, typename T>
struct gb300_kind;
template <>
struct gb300_kind<std::uint32_t, void> : std::integral_constant<int, SG_SET_U32>
{
};
template <>
struct gb300_kind<std::uint64_t, void> : std::integral_constant<int, SG_SET_U64>
{
};
template <>
struct gb300_kind<std::uint64_t, std::uint32_t> : std::integral_constant<int, SG_MAP_U64_U32>
{
};
template <>
struct gb300_kind<std::uint64_t, std::uint64_t> : std::integral_constant<int, SG_MAP_U64_U64>
{
};
template <>
struct gb300_kind<std::uint32_t, std::uint32_t> : std::integral_constant<int, SG_MAP_U32_U32>
{
};
template <>
struct gb300_kind<std::uint32_t, std::uint64_t> : std::integral_constant<int, SG_MAP_U32_U64>
{
};

// Shared implementation of unordered_map / unordered_set (src/stdgpu/impl/unordered_base.cuh:56-583).
template <typename Key, typename T, typename Value, typename Derived>
class gb300_unordered
{
public:
    static constexpr int kind = gb300_kind<Key, T>::value;
    using key_type = Key;
    using value_type = Value;
    using index_type = index_t;
    using iterator = value_type*;
    using const_iterator = const value_type*;
    using ref_type = sg::unordered_ref<kind>;

    static_assert(sizeof(Value) == sg::detail::kind_consts<kind>::slot_bytes, "value_type layout");

    // createDeviceObject(capacity): src/stdgpu/impl/unordered_base_detail.cuh:1254-1308
    static Derived
    createDeviceObject(const index_t& capacity)
    {
        return createDeviceObject(execution::device, capacity);
    }

    static Derived
    createDeviceObject(execution::device_policy policy, const index_t& capacity)
    {
        Derived d;
        gb300_check(sg_unordered_create(kind, capacity, policy.stream, &d._handle), "createDeviceObject");
        gb300_check(sg_unordered_view_of(d._handle, &d._view), "createDeviceObject");
        gb300_check(cudaMalloc(&d._range, sizeof(std::int32_t) * (d._view.total_count + 2)) == cudaSuccess
                            ? SG_OK
                            : SG_ERR_OOM,
                    "createDeviceObject");
        return d;
    }

    // createDeviceObject(capacity, allocator): every device block of the object from `alloc`
    static Derived
    create_with_allocator(execution::device_policy policy, const index_t& capacity, const sg_allocator& alloc)
    {
        Derived d;
        const sg_status st = sg_unordered_create_with_allocator(kind, capacity, 0, &alloc, policy.stream, &d._handle);
        if (st != SG_OK && alloc.release_ctx != nullptr)
        {
            alloc.release_ctx(alloc.ctx);
        }
        gb300_check(st, "createDeviceObject");
        d._alloc = alloc;
        gb300_check(sg_unordered_view_of(d._handle, &d._view), "createDeviceObject");
        d._range = own_alloc<std::int32_t>(alloc, sizeof(std::int32_t) * (d._view.total_count + 2));
        gb300_check(d._range != nullptr ? SG_OK : SG_ERR_OOM, "createDeviceObject");
        return d;
    }

    // destroyDeviceObject: src/stdgpu/impl/unordered_base_detail.cuh:1310-1348
    static void
    destroyDeviceObject(Derived& d)
    {
        destroyDeviceObject(execution::device, d);
    }

    static void
    destroyDeviceObject(execution::device_policy, Derived& d)
    {
        if (d._handle != nullptr)
        {
            if (d._alloc.alloc != nullptr)
            {
                cudaDeviceSynchronize();
                d._alloc.release(d._range, d._alloc.ctx); // before the table drops the allocator's context
            }
            else
            {
                cudaFree(d._range);
            }
            gb300_check(sg_unordered_destroy(d._handle), "destroyDeviceObject");
        }
        d._handle = nullptr;
        d._range = nullptr;
        d._view = sg_unordered_view{};
        d._alloc = sg_allocator{};
    }

    // Not in the reference: the excess-list accounting switch of an empty object
    // (sg_unordered_set_excess_accounting; on by default up to max_size() 2^20).  Off, the object takes keys
    // until no slot is free instead of refusing them where the reference's excess list runs out.  Copies made
    // before the switch keep the old device view.
    void
    set_excess_accounting(bool on)
    {
        gb300_check(sg_unordered_set_excess_accounting(_handle, on ? 1 : 0, nullptr), "set_excess_accounting");
        gb300_check(sg_unordered_view_of(_handle, &_view), "set_excess_accounting");
    }

    // insert(begin, end) over value_type elements: unordered_base_detail.cuh:996-1017
    void
    insert(const value_type* begin, const value_type* end)
    {
        insert(execution::device, begin, end);
    }

    void
    insert(execution::device_policy policy, const value_type* begin, const value_type* end)
    {
        gb300_check(sg_unordered_insert(_handle, begin, static_cast<int64_t>(end - begin), nullptr, policy.stream),
                    "insert");
    }

    // erase(begin, end) over keys: unordered_base_detail.cuh:1045-1066
    void
    erase(const key_type* begin, const key_type* end)
    {
        erase(execution::device, begin, end);
    }

    void
    erase(execution::device_policy policy, const key_type* begin, const key_type* end)
    {
        gb300_check(sg_unordered_erase(_handle, begin, static_cast<int64_t>(end - begin), nullptr, policy.stream),
                    "erase");
    }

    // size() / empty() / full(): unordered_base_detail.cuh:1078-1132 (host side, synchronising)
    index_t
    size(execution::device_policy policy = execution::device) const
    {
        if (_handle == nullptr)
        {
            return 0; // a default-constructed object holds nothing, as in the reference
        }
        int64_t n = 0;
        gb300_check(sg_unordered_size(_handle, policy.stream, &n), "size");
        return static_cast<index_t>(n);
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
        return static_cast<index_t>(_view.total_count);
    }

    __host__ __device__ index_t
    bucket_count() const
    {
        return static_cast<index_t>(_view.bucket_count);
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

    void
    clear(execution::device_policy policy = execution::device)
    {
        gb300_check(sg_unordered_clear(_handle, policy.stream), "clear");
    }

    bool
    valid(execution::device_policy policy = execution::device) const
    {
        if (_handle == nullptr)
        {
            return true; // an empty handle is valid, as in the reference
        }
        int32_t ok = 0;
        gb300_check(sg_unordered_valid(_handle, policy.stream, &ok), "valid");
        return ok != 0;
    }

    // device_range(): unordered_base_detail.cuh:160-208
    device_indexed_range<value_type>
    device_range(execution::device_policy policy = execution::device)
    {
        int64_t n = 0;
        gb300_check(sg_unordered_device_range(_handle, _range, policy.stream, &n), "device_range");
        return device_indexed_range<value_type>{ _range, static_cast<index_t>(n), begin_host() };
    }

    // bucket(key): host and device (unordered_base_detail.cuh:547-564)
    __host__ __device__ index_t
    bucket(const key_type& key) const
    {
        return static_cast<index_t>(sg::detail::fibonacci_bucket(static_cast<std::uint64_t>(key), _view.bucket_bits));
    }

    // ---- device members (unordered_base_detail.cuh:566-706, 958-1043)
    __device__ iterator
    begin() const
    {
        return static_cast<value_type*>(_view.slots);
    }

    __device__ iterator
    end() const
    {
        return begin() + max_size();
    }

    __device__ index_t
    bucket_size(index_t n) const
    {
        return static_cast<index_t>(ref_type{ _view }.bucket_size(n));
    }

    __device__ iterator
    find(const key_type& key) const
    {
        const int64_t s = ref_type{ _view }.find_slot(key);
        return s >= 0 ? begin() + s : end();
    }

    __device__ bool
    contains(const key_type& key) const
    {
        return ref_type{ _view }.contains(key);
    }

    __device__ index_t
    count(const key_type& key) const
    {
        return contains(key) ? 1 : 0;
    }

    __device__ index_t
    erase(const key_type& key) const
    {
        return static_cast<index_t>(ref_type{ _view }.erase(key));
    }

    __host__ __device__ bool
    is_null() const
    {
        return _view.slots == nullptr;
    }

protected:
    __host__ __device__ value_type*
    begin_host() const
    {
        return static_cast<value_type*>(_view.slots);
    }

    __device__ pair<iterator, bool>
    insert_impl(const key_type& key, typename ref_type::mapped_type mapped) const
    {
        const int64_t s = ref_type{ _view }.insert_slot(key, mapped);
        return s >= 0 ? pair<iterator, bool>(begin() + s, true) : pair<iterator, bool>(end(), false);
    }

    sg_unordered* _handle = nullptr;
    sg_unordered_view _view{};
    std::int32_t* _range = nullptr;
    sg_allocator _alloc{}; // the object's own allocator (createDeviceObject(capacity, allocator)), or none
};
} // namespace detail

namespace detail
{
// unordered_map<Key, T> for 4/8-byte unsigned integer Key and T with the identity hash.
template <typename Key, typename T, typename Derived>
class native_map : public gb300_unordered<Key, T, pair<const Key, T>, Derived>
{
    using base = gb300_unordered<Key, T, pair<const Key, T>, Derived>;

public:
    using mapped_type = T;
    using typename base::iterator;
    using typename base::key_type;
    using typename base::value_type;
    using base::erase;
    using base::insert;

    // insert(value) / emplace(args...) (device): unordered_base_detail.cuh:958-994
    __device__ pair<iterator, bool>
    insert(const value_type& value) const
    {
        return this->insert_impl(value.first, value.second);
    }

    __device__ pair<iterator, bool>
    emplace(const Key& key, const T& mapped) const
    {
        return this->insert_impl(key, mapped);
    }
};

// unordered_set<Key> for 4/8-byte unsigned integer Key with the identity hash.
template <typename Key, typename Derived>
class native_set : public gb300_unordered<Key, void, Key, Derived>
{
    using base = gb300_unordered<Key, void, Key, Derived>;

public:
    using typename base::iterator;
    using typename base::key_type;
    using typename base::value_type;
    using base::erase;
    using base::insert;

    __device__ pair<iterator, bool>
    insert(const value_type& key) const
    {
        return this->insert_impl(key, typename base::ref_type::mapped_type{});
    }

    __device__ pair<iterator, bool>
    emplace(const Key& key) const
    {
        return this->insert_impl(key, typename base::ref_type::mapped_type{});
    }
};
} // namespace detail
} // namespace stdgpu

#include "custom_key.cuh"
#include "wide_key.cuh"

namespace stdgpu
{
namespace detail
{
// Which storage an element type takes: the library's precompiled kinds (integer keys with the identity hash
// and 4/8-byte unsigned mapped integers), the word-keyed custom path (any trivially copyable key of at most 8
// bytes with a trivially copyable 4/8-byte mapped type), or the wide path of wide_key.cuh (everything else:
// keys of 9-16 bytes, other mapped types, types with destructors).
template <typename T>
struct mapped_fits_word
  : std::integral_constant<bool, (sizeof(T) == 4 || sizeof(T) == 8) && std::is_trivially_copyable<T>::value>
{
};
template <>
struct mapped_fits_word<void> : std::true_type
{
};

template <typename Key, typename T, typename Hash>
struct is_native_table
  : std::integral_constant<bool, is_native_key<Key, Hash>::value &&
                                         (std::is_void<T>::value || std::is_same<T, std::uint32_t>::value ||
                                          std::is_same<T, std::uint64_t>::value)>
{
};

template <typename Key, typename T>
struct fits_word_table
  : std::integral_constant<bool, sizeof(Key) <= 8 && std::is_trivially_copyable<Key>::value &&
                                         mapped_fits_word<T>::value>
{
};

// Whether keys may compare by their bytes: the default comparison (equal_to<Key>, equal_to<void>,
// std::equal_to<Key>) of a key type whose equal values have equal object bytes (integers, enums, pointers
// and padding-free aggregates of them; not floating point, not types with padding).  Such keys use the
// library's kernels; every other key compares through KeyEqual in the header tables of wide_key.cuh.  A
// class key compared by default must have an operator== that compares all of its members.
template <typename Key, typename KeyEqual>
struct bytes_compare
  : std::integral_constant<bool, (std::is_same<KeyEqual, equal_to<Key>>::value ||
                                  std::is_same<KeyEqual, equal_to<void>>::value ||
                                  std::is_same<KeyEqual, std::equal_to<Key>>::value) &&
                                         std::has_unique_object_representations<Key>::value>
{
};

// The wide tables' comparison for KeyEqual: void (bytes) where bytes_compare holds.
template <typename Key, typename KeyEqual>
using wide_key_equal = std::conditional_t<bytes_compare<Key, KeyEqual>::value, void, KeyEqual>;

// Storage of unordered_map<Key, T, Hash, KeyEqual> / unordered_set (T = void): the library's kinds, the
// word-keyed custom path, or the wide header tables.
template <typename Key, typename T, typename Hash, typename KeyEqual, typename Derived>
using map_storage = std::conditional_t<
        is_native_table<Key, T, Hash>::value && bytes_compare<Key, KeyEqual>::value, native_map<Key, T, Derived>,
        std::conditional_t<fits_word_table<Key, T>::value && bytes_compare<Key, KeyEqual>::value,
                           custom_map<Key, T, Hash, Derived>,
                           wide_map<Key, T, Hash, Derived, wide_key_equal<Key, KeyEqual>>>>;
template <typename Key, typename Hash, typename KeyEqual, typename Derived>
using set_storage = std::conditional_t<
        is_native_table<Key, void, Hash>::value && bytes_compare<Key, KeyEqual>::value, native_set<Key, Derived>,
        std::conditional_t<fits_word_table<Key, void>::value && bytes_compare<Key, KeyEqual>::value,
                           custom_set<Key, Hash, Derived>, wide_set<Key, Hash, Derived, wide_key_equal<Key, KeyEqual>>>>;
} // namespace detail
} // namespace stdgpu

namespace stdgpu
{

// stdgpu::unordered_map<Key, T, Hash, KeyEqual>: integer keys with the default hash and integer mapped values
// use the library's precompiled kernels; other keys of at most 8 bytes (short3, vec3int16, packed coordinates)
// with a user Hash and a 4/8-byte mapped type go through the word-keyed path of custom_key.cuh; every other
// element type (a 3 x int32 key, an empty or 16-byte mapped type, a type with a destructor) through
// wide_key.cuh.  Keys compared by a user KeyEqual, or whose bytes do not decide their equality (floating
// point, padding), also take wide_key.cuh, which calls KeyEqual on every probe (detail::bytes_compare).
template <typename Key, typename T, typename Hash = hash<Key>, typename KeyEqual = equal_to<Key>,
          typename Allocator = safe_device_allocator<pair<const Key, T>>>
class unordered_map
  : public detail::map_storage<Key, T, Hash, KeyEqual, unordered_map<Key, T, Hash, KeyEqual, Allocator>>
{
    using base = detail::map_storage<Key, T, Hash, KeyEqual, unordered_map>;

public:
    using key_equal = KeyEqual;
    using hasher = Hash;
    using allocator_type = Allocator;
    using base::createDeviceObject;

    // createDeviceObject(capacity, allocator) (src/stdgpu/impl/unordered_map_detail.cuh): the allocator is kept
    // and returned by get_allocator()
    static unordered_map
    createDeviceObject(const index_t& capacity, const Allocator& allocator)
    {
        return createDeviceObject(execution::device, capacity, allocator);
    }

    static unordered_map
    createDeviceObject(execution::device_policy policy, const index_t& capacity, const Allocator& allocator)
    {
        unordered_map m = detail::is_safe_device_allocator<Allocator>::value
                                  ? base::createDeviceObject(policy, capacity)
                                  : base::create_with_allocator(policy, capacity,
                                                                detail::allocator_bridge<Allocator>::make(allocator));
        m._allocator = allocator;
        return m;
    }

    allocator_type
    get_allocator() const noexcept
    {
        return _allocator;
    }

    // hash_function() / key_eq() (src/stdgpu/impl/unordered_base_detail.cuh:1178-1190)
    __host__ __device__ hasher
    hash_function() const
    {
        return hasher{};
    }

    __host__ __device__ key_equal
    key_eq() const
    {
        return key_equal{};
    }

private:
    Allocator _allocator{};
};

// stdgpu::unordered_set<Key, Hash>
template <typename Key, typename Hash = hash<Key>, typename KeyEqual = equal_to<Key>,
          typename Allocator = safe_device_allocator<Key>>
class unordered_set : public detail::set_storage<Key, Hash, KeyEqual, unordered_set<Key, Hash, KeyEqual, Allocator>>
{
    using base = detail::set_storage<Key, Hash, KeyEqual, unordered_set>;

public:
    using key_equal = KeyEqual;
    using hasher = Hash;
    using allocator_type = Allocator;
    using base::createDeviceObject;

    static unordered_set
    createDeviceObject(const index_t& capacity, const Allocator& allocator)
    {
        return createDeviceObject(execution::device, capacity, allocator);
    }

    static unordered_set
    createDeviceObject(execution::device_policy policy, const index_t& capacity, const Allocator& allocator)
    {
        unordered_set m = detail::is_safe_device_allocator<Allocator>::value
                                  ? base::createDeviceObject(policy, capacity)
                                  : base::create_with_allocator(policy, capacity,
                                                                detail::allocator_bridge<Allocator>::make(allocator));
        m._allocator = allocator;
        return m;
    }

    allocator_type
    get_allocator() const noexcept
    {
        return _allocator;
    }

    __host__ __device__ hasher
    hash_function() const
    {
        return hasher{};
    }

    __host__ __device__ key_equal
    key_eq() const
    {
        return key_equal{};
    }

private:
    Allocator _allocator{};
};

// A contiguous device range [begin, begin + count): device_range() of vector and deque.
template <typename T>
struct device_range_of
{
    T* first = nullptr;
    index_t count = 0;

    __host__ __device__ index_t
    size() const
    {
        return count;
    }
    __host__ __device__ T*
    begin() const
    {
        return first;
    }
    __host__ __device__ T*
    end() const
    {
        return first + count;
    }
    __device__ T&
    operator[](index_t i) const
    {
        return first[i];
    }
};

// stdgpu::vector<T> (src/stdgpu/vector.cuh) for 4/8-byte T: the reference's host calls over the C ABI and
// its device calls on the vector's view.  Device push_back is warp-aggregated like the bulk kernel, and
// device push_back and pop_back may share a launch: each takes its position from the counter and then
// waits (bounded) on the slot's word until the slot is free (push) or written (pop) -- the reference's
// per-slot occupied bit (vector_detail.cuh:181-299), kept as (epoch << 1) | occupied so that bulk calls,
// which end by advancing the epoch, never touch the slot words (sg_vector_sync).  Device calls and bulk
// calls on one vector must not run at the same time.
template <typename T, typename Allocator = safe_device_allocator<T>>
class vector
{
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");

public:
    using value_type = T;
    using allocator_type = Allocator;

    allocator_type
    get_allocator() const noexcept
    {
        return _allocator;
    }

    // createDeviceObject(capacity, allocator): with an allocator other than the default, every device block of
    // the vector comes from it (detail::allocator_bridge); get_allocator() returns it
    static vector
    createDeviceObject(const index_t& capacity, const Allocator& allocator)
    {
        vector x;
        if constexpr (detail::is_safe_device_allocator<Allocator>::value)
        {
            x = createDeviceObject(execution::device, capacity);
        }
        else
        {
            const sg_allocator a = detail::allocator_bridge<Allocator>::make(allocator);
            const sg_status st = sg_vector_create_with_allocator(sizeof(T), capacity, &a, &x._handle);
            if (st != SG_OK)
            {
                a.release_ctx(a.ctx);
            }
            detail::gb300_check(st, "vector::createDeviceObject");
            detail::gb300_check(sg_vector_view_of(x._handle, &x._view), "vector::createDeviceObject");
        }
        x._allocator = allocator;
        return x;
    }

    static vector
    createDeviceObject(const index_t& capacity)
    {
        return createDeviceObject(execution::device, capacity);
    }

    static vector
    createDeviceObject(execution::device_policy, const index_t& capacity)
    {
        vector v;
        detail::gb300_check(sg_vector_create(sizeof(T), capacity, &v._handle), "vector::createDeviceObject");
        detail::gb300_check(sg_vector_view_of(v._handle, &v._view), "vector::createDeviceObject");
        return v;
    }

    static void
    destroyDeviceObject(vector& v)
    {
        destroyDeviceObject(execution::device, v);
    }

    static void
    destroyDeviceObject(execution::device_policy, vector& v)
    {
        if (v._handle != nullptr)
        {
            detail::gb300_check(sg_vector_destroy(v._handle), "vector::destroyDeviceObject");
        }
        v._handle = nullptr;
        v._view = sg_vector_view{};
    }

    index_t
    size(execution::device_policy policy = execution::device) const
    {
        if (_handle == nullptr)
        {
            return 0;
        }
        int64_t n = 0;
        detail::gb300_check(sg_vector_size(_handle, policy.stream, &n), "vector::size");
        return static_cast<index_t>(n);
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
    capacity() const
    {
        return static_cast<index_t>(_view.capacity);
    }

    __host__ __device__ index_t
    max_size() const noexcept
    {
        return capacity();
    }

    __host__ __device__ T*
    data() const
    {
        return static_cast<T*>(_view.data);
    }

    void
    clear(execution::device_policy policy = execution::device)
    {
        detail::gb300_check(sg_vector_clear(_handle, policy.stream), "vector::clear");
    }

    // valid() (src/stdgpu/impl/vector_detail.cuh:614-640): the element count lies in [0, capacity()]
    bool
    valid(execution::device_policy policy = execution::device) const
    {
        if (_handle == nullptr)
        {
            return true;
        }
        long long n = -1;
        sg_vector_sync sy{};
        const bool ok = cudaMemcpyAsync(&n, _view.size, sizeof(n), cudaMemcpyDeviceToHost, policy.stream) == cudaSuccess &&
                        cudaMemcpyAsync(&sy, _view.sync, sizeof(sy), cudaMemcpyDeviceToHost, policy.stream) == cudaSuccess &&
                        cudaStreamSynchronize(policy.stream) == cudaSuccess;
        detail::gb300_check(ok ? SG_OK : SG_ERR_CUDA, "vector::valid");
        return n >= 0 && n <= _view.capacity && sy.error == 0u;
    }

    // device_begin() / device_end() / device_range(): the stored elements [data(), data() + size())
    T*
    device_begin() const
    {
        return data();
    }

    T*
    device_end(execution::device_policy policy = execution::device) const
    {
        return data() + size(policy);
    }

    device_range_of<T>
    device_range(execution::device_policy policy = execution::device) const
    {
        return device_range_of<T>{ data(), size(policy) };
    }

    // insert(position, begin, end) (src/stdgpu/impl/vector_detail.cuh:372-410): position must be device_end();
    // values that would not fit are not inserted at all, as in the reference.
    void
    insert(const T* position, const T* begin, const T* end)
    {
        insert(execution::device, position, begin, end);
    }

    void
    insert(execution::device_policy policy, const T* position, const T* begin, const T* end)
    {
        if (position != device_end(policy))
        {
            detail::gb300_check(SG_ERR_BAD_ARG, "vector::insert (only at device_end())");
            return;
        }
        const sg_status st = sg_vector_insert(_handle, begin, end - begin, policy.stream);
        detail::gb300_check(st == SG_ERR_FULL ? SG_OK : st, "vector::insert");
    }

    // erase(begin, end) (src/stdgpu/impl/vector_detail.cuh:418-450): a suffix ending at device_end()
    void
    erase(const T* begin, const T* end)
    {
        erase(execution::device, begin, end);
    }

    void
    erase(execution::device_policy policy, const T* begin, const T* end)
    {
        if (end != device_end(policy) || begin > end || begin < device_begin())
        {
            detail::gb300_check(SG_ERR_BAD_ARG, "vector::erase (only a suffix ending at device_end())");
            return;
        }
        detail::gb300_check(sg_vector_erase(_handle, end - begin, policy.stream), "vector::erase");
    }

    // Slot word protocol of the device calls.  A word of another epoch has not been touched since the last
    // bulk call: its slot is occupied exactly when it lies below the size that call left.
    __device__ bool
    slot_occupied(long long pos, uint32_t epoch, long long base) const
    {
        unsigned short w;
        asm volatile("ld.acquire.gpu.global.u16 %0, [%1];"
                     : "=h"(w)
                     : "l"(static_cast<unsigned short*>(_view.slot_state) + pos)
                     : "memory");
        return (static_cast<uint32_t>(w) >> 1) == epoch ? (w & 1u) != 0u : pos < base;
    }

    __device__ void
    set_slot(long long pos, uint32_t epoch, bool occupied) const
    {
        const unsigned short w = static_cast<unsigned short>((epoch << 1) | (occupied ? 1u : 0u));
        asm volatile("st.release.gpu.global.u16 [%0], %1;" ::"l"(static_cast<unsigned short*>(_view.slot_state) + pos),
                     "h"(w)
                     : "memory");
    }

    // Waits until slot pos is occupied (want == true) or free; false when the wait ran out (~1 s), which sets
    // the error bit that valid() reports.
    __device__ bool
    wait_slot(long long pos, bool want, uint32_t epoch, long long base) const
    {
        unsigned backoff = 32;
        for (long long polls = 0; polls < ::sg::detail::kWaitLimit; ++polls)
        {
            if (slot_occupied(pos, epoch, base) == want)
            {
                return true;
            }
            __nanosleep(backoff);
            backoff = backoff < 256 ? backoff * 2 : 256;
        }
        atomicOr(&static_cast<sg_vector_sync*>(_view.sync)->error, 1u);
        return false;
    }

    __device__ void
    sync_state(uint32_t& epoch, long long& base) const
    {
        const sg_vector_sync* sy = static_cast<const sg_vector_sync*>(_view.sync);
        epoch = *reinterpret_cast<const volatile uint32_t*>(&sy->epoch);
        base = *reinterpret_cast<const volatile long long*>(&sy->base_size);
    }

    // Device push_back (src/stdgpu/impl/vector_detail.cuh:181-238): the calling lanes that are active
    // together reserve their positions with one atomic per warp; each then waits until its slot is free (a
    // pop_back of the same launch may still be reading it) and writes.
    __device__ bool
    push_back(const T& element) const
    {
        const unsigned active = __activemask();
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(active) - 1;
        unsigned lt;
        asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
        long long* size = static_cast<long long*>(_view.size);
        long long base = -1;
        if (lane == leader)
        {
            const long long cur = *reinterpret_cast<volatile long long*>(size);
            base = cur >= _view.capacity ? -1
                                         : static_cast<long long>(atomicAdd(reinterpret_cast<unsigned long long*>(size),
                                                                            static_cast<unsigned long long>(__popc(active))));
        }
        base = __shfl_sync(active, base, leader);
        const long long pos = base + __popc(active & lt);
        if (base < 0 || pos >= _view.capacity)
        {
            return false;
        }
        uint32_t epoch;
        long long start;
        sync_state(epoch, start);
        if (!wait_slot(pos, false, epoch, start))
        {
            return false;
        }
        data()[pos] = element;
        set_slot(pos, epoch, true);
        return true;
    }

    template <typename... Args>
    __device__ bool
    emplace_back(Args&&... args) const
    {
        return push_back(T(static_cast<Args&&>(args)...));
    }

    // Device pop_back (src/stdgpu/impl/vector_detail.cuh:240-299): takes the last element, or fails on an
    // empty vector.  The count is taken down with a bounded compare-and-swap loop; the pop then waits until
    // its slot is written (a push_back of the same launch may not have stored it yet), reads it and frees it.
    __device__ pair<T, bool>
    pop_back() const
    {
        unsigned long long* size = static_cast<unsigned long long*>(_view.size);
        long long cur = *reinterpret_cast<volatile long long*>(size);
        for (int tries = 0; tries < (1 << 20); ++tries)
        {
            if (cur <= 0)
            {
                return pair<T, bool>(T{}, false);
            }
            const long long n = cur > _view.capacity ? _view.capacity : cur;
            const long long seen = static_cast<long long>(atomicCAS(size, static_cast<unsigned long long>(cur),
                                                                    static_cast<unsigned long long>(n - 1)));
            if (seen == cur)
            {
                uint32_t epoch;
                long long start;
                sync_state(epoch, start);
                if (!wait_slot(n - 1, true, epoch, start))
                {
                    return pair<T, bool>(T{}, false);
                }
                const T x = *reinterpret_cast<volatile T*>(data() + (n - 1));
                set_slot(n - 1, epoch, false);
                return pair<T, bool>(x, true);
            }
            cur = seen;
        }
        return pair<T, bool>(T{}, false);
    }

    // element access (src/stdgpu/impl/vector_detail.cuh:113-175: at, operator[], front, back)
    __device__ T&
    at(index_t n) const
    {
        return data()[n];
    }

    __device__ T&
    operator[](index_t n) const
    {
        return data()[n];
    }

    __device__ T&
    front() const
    {
        return data()[0];
    }

    __device__ T&
    back() const
    {
        const long long n = *reinterpret_cast<volatile long long*>(_view.size);
        return data()[(n > _view.capacity ? _view.capacity : n) - 1];
    }

private:
    sg_vector* _handle = nullptr;
    sg_vector_view _view{};
    Allocator _allocator{};
};

// stdgpu::deque<T> (src/stdgpu/deque.cuh) for 4/8-byte T.  Device push_back, push_front, pop_front and
// pop_back may run in any mix in one kernel: each takes its ticket from the counters (size guards the
// capacity, avail the elements) and then waits on its slot's word until the slot is free (push) or written
// (pop), the reference's per-slot occupied bit (deque_detail.cuh:202-446); the waits are bounded (one that
// runs out sets the deque's error bit, which size() reports, and the call fails).  The host bulk calls
// (push_back / pop_front mixes, push_front, pop_back) keep turn words of their own, rebuilt from the tickets
// after device calls ran (sg_deque_sync).  Device calls and bulk calls on one deque must not run at the same
// time.
template <typename T, typename Allocator = safe_device_allocator<T>>
class deque
{
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "4- or 8-byte elements");

public:
    using value_type = T;
    using allocator_type = Allocator;

    allocator_type
    get_allocator() const noexcept
    {
        return _allocator;
    }

    // createDeviceObject(capacity, allocator): with an allocator other than the default, every device block of
    // the deque (its ring, and the array device_range() copies into) comes from it; get_allocator() returns it
    static deque
    createDeviceObject(const index_t& capacity, const Allocator& allocator)
    {
        deque x;
        if constexpr (detail::is_safe_device_allocator<Allocator>::value)
        {
            x = createDeviceObject(execution::device, capacity);
        }
        else
        {
            const sg_allocator a = detail::allocator_bridge<Allocator>::make(allocator);
            const sg_status st = sg_deque_create_with_allocator(sizeof(T), capacity, &a, &x._handle);
            if (st != SG_OK)
            {
                a.release_ctx(a.ctx);
            }
            detail::gb300_check(st, "deque::createDeviceObject");
            detail::gb300_check(sg_deque_view_of(x._handle, &x._view), "deque::createDeviceObject");
            x._alloc = sg_allocator{ a.alloc, a.release, a.ctx, nullptr }; // the deque's handle owns the context
        }
        x._allocator = allocator;
        return x;
    }

    static deque
    createDeviceObject(const index_t& capacity)
    {
        return createDeviceObject(execution::device, capacity);
    }

    static deque
    createDeviceObject(execution::device_policy, const index_t& capacity)
    {
        deque d;
        detail::gb300_check(sg_deque_create(sizeof(T), capacity, &d._handle), "deque::createDeviceObject");
        detail::gb300_check(sg_deque_view_of(d._handle, &d._view), "deque::createDeviceObject");
        return d;
    }

    static void
    destroyDeviceObject(deque& d)
    {
        destroyDeviceObject(execution::device, d);
    }

    static void
    destroyDeviceObject(execution::device_policy, deque& d)
    {
        if (d._range != nullptr && d._alloc.alloc != nullptr)
        {
            cudaDeviceSynchronize();
            d._alloc.release(d._range, d._alloc.ctx); // before the handle drops the allocator's context
        }
        else
        {
            cudaFree(d._range);
        }
        if (d._handle != nullptr)
        {
            detail::gb300_check(sg_deque_destroy(d._handle), "deque::destroyDeviceObject");
        }
        d._handle = nullptr;
        d._view = sg_deque_view{};
        d._range = nullptr;
        d._alloc = sg_allocator{};
    }

    index_t
    size(execution::device_policy policy = execution::device) const
    {
        if (_handle == nullptr)
        {
            return 0;
        }
        int64_t n = 0;
        detail::gb300_check(sg_deque_size(_handle, policy.stream, &n), "deque::size");
        return static_cast<index_t>(n);
    }

    bool
    empty(execution::device_policy policy = execution::device) const
    {
        return size(policy) == 0;
    }

    bool
    full(execution::device_policy policy = execution::device) const
    {
        return size(policy) == capacity();
    }

    __host__ __device__ index_t
    capacity() const
    {
        return static_cast<index_t>(_view.capacity);
    }

    __host__ __device__ index_t
    max_size() const noexcept
    {
        return capacity();
    }

    // valid() (src/stdgpu/impl/deque_detail.cuh:635-660): the count lies in [0, capacity()] and no bounded wait
    // of a device call has given up
    bool
    valid(execution::device_policy policy = execution::device) const
    {
        if (_handle == nullptr)
        {
            return true;
        }
        int64_t n = 0;
        const sg_status st = sg_deque_size(_handle, policy.stream, &n);
        return st == SG_OK && n >= 0 && n <= _view.capacity;
    }

    // device_range(): the stored elements front to back.  Unlike the reference's range, which indexes the
    // deque's own storage, this is a copy in an array the object keeps (allocated by the first call).
    device_range_of<T>
    device_range(execution::device_policy policy = execution::device)
    {
        if (_range == nullptr && _view.capacity > 0)
        {
            if (_alloc.alloc != nullptr)
            {
                _range = detail::own_alloc<T>(_alloc, sizeof(T) * _view.capacity);
            }
            else if (cudaMalloc(&_range, sizeof(T) * _view.capacity) != cudaSuccess)
            {
                _range = nullptr;
            }
            detail::gb300_check(_range != nullptr ? SG_OK : SG_ERR_OOM, "deque::device_range");
        }
        int64_t n = 0;
        detail::gb300_check(sg_deque_copy_out(_handle, _range, policy.stream, &n), "deque::device_range");
        return device_range_of<T>{ _range, static_cast<index_t>(n) };
    }

    void
    clear(execution::device_policy policy = execution::device)
    {
        detail::gb300_check(sg_deque_clear(_handle, policy.stream), "deque::clear");
    }

    // data() (src/stdgpu/deque.cuh): the ring's storage; element i sits at slot (front ticket + i) mod
    // capacity(), which is i on a deque that never wrapped or moved its front
    __host__ __device__ T*
    data() const
    {
        return static_cast<T*>(_view.data);
    }

    // the C-ABI handle, for the sg_deque_* entry points (for example sg_deque_ops, a bulk push_back /
    // pop_front mix)
    sg_deque*
    native_handle() const noexcept
    {
        return _handle;
    }

    // host bulk forms (device pointers): push_front / pop_back of n elements, as sequences of calls
    void
    push_front(const T* values, index_t n, std::uint8_t* ok = nullptr,
               execution::device_policy policy = execution::device)
    {
        detail::gb300_check(sg_deque_push_front(_handle, values, n, ok, policy.stream), "deque::push_front");
    }

    void
    pop_back(index_t n, T* popped, std::uint8_t* ok = nullptr, execution::device_policy policy = execution::device)
    {
        detail::gb300_check(sg_deque_pop_back(_handle, n, popped, ok, policy.stream), "deque::pop_back");
    }

private:
    // Slot words of the device calls: (epoch << 1) | occupied.  A word of another epoch has not been touched
    // since the last bulk call; its slot is occupied exactly when the ticket mapping to it lay in
    // [base_begin, base_end) after that call.
    __device__ bool
    slot_occupied(long long pos, uint32_t epoch, unsigned long long b0, unsigned long long e0) const
    {
        unsigned short w;
        asm volatile("ld.acquire.gpu.global.u16 %0, [%1];"
                     : "=h"(w)
                     : "l"(static_cast<unsigned short*>(_view.slot_state) + pos)
                     : "memory");
        if ((static_cast<uint32_t>(w) >> 1) == epoch)
        {
            return (w & 1u) != 0u;
        }
        const unsigned long long cap = static_cast<unsigned long long>(_view.capacity);
        const unsigned long long from_b = (static_cast<unsigned long long>(pos) + cap - b0 % cap) % cap;
        return from_b < e0 - b0;
    }

    __device__ void
    set_slot(long long pos, uint32_t epoch, bool occupied) const
    {
        const unsigned short w = static_cast<unsigned short>((epoch << 1) | (occupied ? 1u : 0u));
        asm volatile("st.release.gpu.global.u16 [%0], %1;" ::"l"(static_cast<unsigned short*>(_view.slot_state) + pos),
                     "h"(w)
                     : "memory");
    }

    // Waits until the slot is occupied (want) or free; false after ~1 s, which sets the deque's error bit
    // (size() then reports SG_ERR_RETRY_EXHAUSTED).
    __device__ bool
    wait_slot(long long pos, bool want) const
    {
        const sg_deque_sync* sy = static_cast<const sg_deque_sync*>(_view.sync);
        const uint32_t epoch = *reinterpret_cast<const volatile uint32_t*>(&sy->epoch);
        const unsigned long long b0 = *reinterpret_cast<const volatile unsigned long long*>(&sy->base_begin);
        const unsigned long long e0 = *reinterpret_cast<const volatile unsigned long long*>(&sy->base_end);
        unsigned backoff = 32;
        for (long long polls = 0; polls < ::sg::detail::kWaitLimit; ++polls)
        {
            if (slot_occupied(pos, epoch, b0, e0) == want)
            {
                return true;
            }
            __nanosleep(backoff);
            backoff = backoff < 256 ? backoff * 2 : 256;
        }
        atomicOr(&counters()->error, ::sg::detail::kDequeErrWait);
        return false;
    }

    __device__ uint32_t
    current_epoch() const
    {
        return *reinterpret_cast<const volatile uint32_t*>(&static_cast<const sg_deque_sync*>(_view.sync)->epoch);
    }

    // the next bulk call must rebuild its turn words
    __device__ void
    mark_dirty() const
    {
        uint32_t* dirty = &static_cast<sg_deque_sync*>(_view.sync)->dirty;
        if (*reinterpret_cast<volatile uint32_t*>(dirty) == 0u)
        {
            atomicExch(dirty, 1u);
        }
    }

    // A push's reservation: size guards the capacity (taken first); false when full.
    __device__ bool
    reserve_push() const
    {
        auto* c = counters();
        const long long cap = _view.capacity;
        if (*reinterpret_cast<volatile long long*>(&c->size) >= cap) // preemptive full() check
        {
            return false;
        }
        if (static_cast<long long>(atomicAdd(reinterpret_cast<unsigned long long*>(&c->size), 1ull)) >= cap)
        {
            atomicAdd(reinterpret_cast<unsigned long long*>(&c->size), ~0ull);
            return false;
        }
        return true;
    }

    // A pop's reservation: avail guards the elements (taken first); false when empty.
    __device__ bool
    reserve_pop() const
    {
        auto* c = counters();
        if (*reinterpret_cast<volatile long long*>(&c->avail) <= 0) // preemptive empty() check
        {
            return false;
        }
        if (static_cast<long long>(atomicAdd(reinterpret_cast<unsigned long long*>(&c->avail), ~0ull)) <= 0)
        {
            atomicAdd(reinterpret_cast<unsigned long long*>(&c->avail), 1ull);
            return false;
        }
        return true;
    }

    __device__ bool
    push_at(unsigned long long tk, const T& element) const
    {
        auto* c = counters();
        const long long pos = static_cast<long long>(tk % static_cast<unsigned long long>(_view.capacity));
        mark_dirty();
        if (!wait_slot(pos, false))
        {
            return false;
        }
        static_cast<T*>(_view.data)[pos] = element;
        set_slot(pos, current_epoch(), true);
        atomicAdd(reinterpret_cast<unsigned long long*>(&c->avail), 1ull);
        return true;
    }

    __device__ pair<T, bool>
    pop_at(unsigned long long tk) const
    {
        auto* c = counters();
        const long long pos = static_cast<long long>(tk % static_cast<unsigned long long>(_view.capacity));
        mark_dirty();
        if (!wait_slot(pos, true))
        {
            return pair<T, bool>(T{}, false);
        }
        const T v = *reinterpret_cast<volatile T*>(static_cast<T*>(_view.data) + pos);
        set_slot(pos, current_epoch(), false);
        atomicAdd(reinterpret_cast<unsigned long long*>(&c->size), ~0ull);
        return pair<T, bool>(v, true);
    }

public:
    // device push_back (src/stdgpu/impl/deque_detail.cuh:202-258): a ticket from end (end moves up), then the
    // slot is written once free
    __device__ bool
    push_back(const T& element) const
    {
        if (!reserve_push())
        {
            return false;
        }
        return push_at(atomicAdd(&counters()->end, 1ull), element);
    }

    // device push_front (src/stdgpu/impl/deque_detail.cuh:315-386): a ticket below begin (begin moves down)
    __device__ bool
    push_front(const T& element) const
    {
        if (!reserve_push())
        {
            return false;
        }
        return push_at(atomicAdd(&counters()->begin, ~0ull) - 1ull, element);
    }

    template <typename... Args>
    __device__ bool
    emplace_front(Args&&... args) const
    {
        return push_front(T(static_cast<Args&&>(args)...));
    }

    // device pop_back (src/stdgpu/impl/deque_detail.cuh:260-313): the ticket below end (end moves down), read
    // once written
    __device__ pair<T, bool>
    pop_back() const
    {
        if (!reserve_pop())
        {
            return pair<T, bool>(T{}, false);
        }
        return pop_at(atomicAdd(&counters()->end, ~0ull) - 1ull);
    }

    template <typename... Args>
    __device__ bool
    emplace_back(Args&&... args) const
    {
        return push_back(T(static_cast<Args&&>(args)...));
    }

    // element access relative to the front (src/stdgpu/impl/deque_detail.cuh:133-192: at, operator[], front,
    // back); valid while no push or pop runs
    __device__ T&
    operator[](index_t n) const
    {
        const auto* c = counters();
        const unsigned long long cap = static_cast<unsigned long long>(_view.capacity);
        return static_cast<T*>(_view.data)[(c->begin + static_cast<unsigned long long>(n)) % cap];
    }

    __device__ T&
    at(index_t n) const
    {
        return (*this)[n];
    }

    __device__ T&
    front() const
    {
        return (*this)[0];
    }

    __device__ T&
    back() const
    {
        const auto* c = counters();
        const unsigned long long cap = static_cast<unsigned long long>(_view.capacity);
        return static_cast<T*>(_view.data)[(c->end + cap - 1) % cap];
    }

    // device pop_front (src/stdgpu/impl/deque_detail.cuh:388-446): the ticket at begin (begin moves up)
    __device__ pair<T, bool>
    pop_front() const
    {
        if (!reserve_pop())
        {
            return pair<T, bool>(T{}, false);
        }
        return pop_at(atomicAdd(&counters()->begin, 1ull));
    }

private:
    __device__ sg::detail::deque_counters*
    counters() const
    {
        return static_cast<sg::detail::deque_counters*>(_view.counters);
    }

    sg_deque* _handle = nullptr;
    sg_deque_view _view{};
    Allocator _allocator{};
    T* _range = nullptr;
    sg_allocator _alloc{}; // the deque's own allocator (createDeviceObject(capacity, allocator)), or none
};

// stdgpu::queue<T> / stack<T> (src/stdgpu/queue.cuh, stack.cuh): adapters over deque.  queue::push / pop
// are push_back / pop_front (device calls, concurrent); stack::push is push_back and stack::pop the host
// bulk pop_back.
template <typename T, typename ContainerT = deque<T>>
class queue
{
public:
    using container_type = ContainerT;
    using value_type = typename ContainerT::value_type;

    static queue
    createDeviceObject(const index_t& capacity)
    {
        return queue{ ContainerT::createDeviceObject(capacity) };
    }
    static void
    destroyDeviceObject(queue& q)
    {
        ContainerT::destroyDeviceObject(q._c);
    }
    __device__ bool
    push(const T& element) const
    {
        return _c.push_back(element);
    }
    __device__ pair<T, bool>
    pop() const
    {
        return _c.pop_front();
    }
    index_t
    size(execution::device_policy policy = execution::device) const
    {
        return _c.size(policy);
    }
    bool
    empty(execution::device_policy policy = execution::device) const
    {
        return _c.empty(policy);
    }

    ContainerT _c;
};

template <typename T, typename ContainerT = deque<T>>
class stack
{
public:
    using container_type = ContainerT;
    using value_type = typename ContainerT::value_type;

    static stack
    createDeviceObject(const index_t& capacity)
    {
        return stack{ ContainerT::createDeviceObject(capacity) };
    }
    static void
    destroyDeviceObject(stack& s)
    {
        ContainerT::destroyDeviceObject(s._c);
    }
    __device__ bool
    push(const T& element) const
    {
        return _c.push_back(element);
    }
    void
    pop(index_t n, T* popped, std::uint8_t* ok = nullptr, execution::device_policy policy = execution::device)
    {
        _c.pop_back(n, popped, ok, policy);
    }
    index_t
    size(execution::device_policy policy = execution::device) const
    {
        return _c.size(policy);
    }

    ContainerT _c;
};

// bitset::count() over raw blocks (src/stdgpu/impl/bitset_detail.cuh:388-404).
inline std::int64_t
bitset_count(const std::uint32_t* blocks, std::int64_t nbits, execution::device_policy policy = execution::device)
{
    std::int64_t n = 0;
    detail::gb300_check(sg_bitset_count(blocks, nbits, policy.stream, &n), "bitset::count");
    return n;
}

} // namespace stdgpu

#endif

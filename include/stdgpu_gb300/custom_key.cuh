// unordered_map<Key, T, Hash> / unordered_set<Key, Hash> for key types other than the integers, with the
// user's Hash functor (the reference's containers take any Key with Hash and KeyEqual,
// src/stdgpu/unordered_map.cuh:70-80, src/stdgpu/unordered_set.cuh:61-69; its own tests use a 3 x int16 key
// with a spatial hash, tests/stdgpu/unordered_map.inc:178-206, and its README a short3 block set).
//
// A key of at most 8 bytes is stored as its object bytes zero-padded to a 4- or 8-byte key word, so the
// table is one of the library's six kinds; keys compare equal when their bytes do (true for short3,
// vec3int16 and packed coordinates, whose members fill the object without padding).  The bucket of a key is
// the fibonacci hashing of Hash(key), as in the reference: bulk calls compute the hashes in a small kernel
// of this header (instantiated in the caller's translation unit with the caller's Hash) and hand them to
// the library's *_hashed entry points; device calls hash inside the caller's kernel.  The mapped type is
// any trivially copyable type of 4 or 8 bytes (an index, a float, a pointer).
//
// Differences from the reference's interface, all forced by the storage of a key as a word: find()
// returns an iterator whose elements are value_type copies (the slot holds the key word, not a Key
// object), and device_range() gives key(i) / mapped(i) instead of value_type references.
#ifndef STDGPU_GB300_CUSTOM_KEY_CUH
#define STDGPU_GB300_CUSTOM_KEY_CUH

#include <cuda_runtime.h>

#include <cstdint>
#include <cstring>
#include <type_traits>

namespace stdgpu
{
namespace detail
{

template <typename Key, typename Hash>
struct is_native_key
  : std::integral_constant<bool, (std::is_same<Key, std::uint32_t>::value || std::is_same<Key, std::uint64_t>::value) &&
                                         std::is_same<Hash, hash<Key>>::value>
{
};

template <typename Key>
using word_of = std::conditional_t<sizeof(Key) <= 4, std::uint32_t, std::uint64_t>;

template <typename T>
struct mapped_word
{
    using type = std::conditional_t<sizeof(T) <= 4, std::uint32_t, std::uint64_t>;
};
template <>
struct mapped_word<void>
{
    using type = void;
};

template <typename W, typename M>
struct word_kind;
template <>
struct word_kind<std::uint32_t, void> : std::integral_constant<int, SG_SET_U32>
{
};
template <>
struct word_kind<std::uint64_t, void> : std::integral_constant<int, SG_SET_U64>
{
};
template <>
struct word_kind<std::uint64_t, std::uint32_t> : std::integral_constant<int, SG_MAP_U64_U32>
{
};
template <>
struct word_kind<std::uint64_t, std::uint64_t> : std::integral_constant<int, SG_MAP_U64_U64>
{
};
template <>
struct word_kind<std::uint32_t, std::uint32_t> : std::integral_constant<int, SG_MAP_U32_U32>
{
};
template <>
struct word_kind<std::uint32_t, std::uint64_t> : std::integral_constant<int, SG_MAP_U32_U64>
{
};

template <typename W, typename X>
__host__ __device__ inline W
to_word(const X& x)
{
    W w = 0;
    std::memcpy(&w, &x, sizeof(X));
    return w;
}

template <typename X, typename W>
__host__ __device__ inline X
from_word(W w)
{
    X x;
    std::memcpy(&x, &w, sizeof(X));
    return x;
}

// Hash of a key word: the user's Hash applied to the Key the word holds.
template <typename Key, typename Hash>
struct word_hash
{
    template <typename W>
    __host__ __device__ std::uint64_t
    operator()(W w) const
    {
        return static_cast<std::uint64_t>(Hash{}(from_word<Key>(w)));
    }
};

// Bulk-call preparation: key words, mapped words and hashes of n elements.
template <typename Key, typename T, typename Hash, typename Value>
__global__ void
k_prepare(const Value* in, std::int64_t n, word_of<Key>* words, typename mapped_word<T>::type* mapped,
          std::uint64_t* hashes)
{
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    for (std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        const Value v = in[i];
        Key key;
        if constexpr (std::is_same<T, void>::value)
        {
            key = v;
        }
        else
        {
            key = v.first;
            mapped[i] = to_word<typename mapped_word<T>::type>(v.second);
        }
        words[i] = to_word<word_of<Key>>(key);
        hashes[i] = static_cast<std::uint64_t>(Hash{}(key));
    }
}

template <typename Key, typename Hash>
__global__ void
k_prepare_keys(const Key* in, std::int64_t n, word_of<Key>* words, std::uint64_t* hashes, bool from_words)
{
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    for (std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        const Key key = from_words ? from_word<Key>(words[i]) : in[i];
        if (!from_words)
        {
            words[i] = to_word<word_of<Key>>(key);
        }
        hashes[i] = static_cast<std::uint64_t>(Hash{}(key));
    }
}

template <int Unused = 0>
__global__ void
k_all_set(const std::uint8_t* flags, std::int64_t n, unsigned int* missing)
{
    const std::int64_t stride = static_cast<std::int64_t>(gridDim.x) * blockDim.x;
    for (std::int64_t i = blockIdx.x * static_cast<std::int64_t>(blockDim.x) + threadIdx.x; i < n; i += stride)
    {
        if (flags[i] == 0)
        {
            atomicAdd(missing, 1u);
        }
    }
}

inline unsigned int
grid_of(std::int64_t n)
{
    const std::int64_t g = (n + 255) / 256;
    return static_cast<unsigned int>(g < 1 ? 1 : (g > 4096 ? 4096 : g));
}

// Stream-ordered scratch for one bulk call.
struct scratch
{
    void* p = nullptr;
    cudaStream_t s = nullptr;
    scratch(std::size_t bytes, cudaStream_t stream)
      : s(stream)
    {
        gb300_check(cudaMallocAsync(&p, bytes > 0 ? bytes : 1, s) == cudaSuccess ? SG_OK : SG_ERR_OOM, "scratch");
    }
    ~scratch() { cudaFreeAsync(p, s); }
    scratch(const scratch&) = delete;
    scratch& operator=(const scratch&) = delete;
};

// The table's own staging buffer for a bulk call (sg_unordered_call_scratch): no allocation per call.
struct table_scratch
{
    void* p = nullptr;
    table_scratch(sg_unordered* h, std::size_t bytes, cudaStream_t s)
    {
        gb300_check(sg_unordered_call_scratch(h, static_cast<std::int64_t>(bytes), s, &p), "scratch");
    }
};

inline std::size_t
align256(std::size_t x)
{
    return (x + 255) / 256 * 256;
}

// Iterator of find(): a slot position; dereferencing gives the slot's element as a value_type copy.
template <typename Key, typename T, typename Value>
struct custom_iterator
{
    using W = word_of<Key>;
    const char* slot = nullptr;
    int slot_bytes = 0;
    int val_offset = 0;

    __device__ Value
    operator*() const
    {
        const W w = *reinterpret_cast<const W*>(slot);
        if constexpr (std::is_same<T, void>::value)
        {
            return from_word<Key>(w);
        }
        else
        {
            using M = typename mapped_word<T>::type;
            const M m = *reinterpret_cast<const M*>(slot + val_offset);
            return Value(from_word<Key>(w), from_word<T>(m));
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

    __host__ __device__ bool
    operator==(const custom_iterator& o) const
    {
        return slot == o.slot;
    }

    __host__ __device__ bool
    operator!=(const custom_iterator& o) const
    {
        return slot != o.slot;
    }
};

// device_range() of a custom-key table: the stored elements through their slot indices.
template <typename Key, typename T>
struct custom_range
{
    using W = word_of<Key>;
    const std::int32_t* indices = nullptr;
    index_t count = 0;
    const char* slots = nullptr;
    int slot_bytes = 0;
    int val_offset = 0;

    __host__ __device__ index_t
    size() const
    {
        return count;
    }

    __device__ Key
    key(index_t i) const
    {
        return from_word<Key>(*reinterpret_cast<const W*>(slots + static_cast<std::int64_t>(indices[i]) * slot_bytes));
    }

    template <typename U = T, typename = std::enable_if_t<!std::is_same<U, void>::value>>
    __device__ U
    mapped(index_t i) const
    {
        using M = typename mapped_word<U>::type;
        return from_word<U>(*reinterpret_cast<const M*>(slots + static_cast<std::int64_t>(indices[i]) * slot_bytes +
                                                        val_offset));
    }
};

template <typename Key, typename T, typename Hash, typename Value, typename Derived>
class custom_unordered
{
    static_assert(sizeof(Key) <= 8, "a custom key type must fit in 8 bytes");
    static_assert(std::is_trivially_copyable<Key>::value, "a custom key type must be trivially copyable");

public:
    using W = word_of<Key>;
    using M = typename mapped_word<T>::type;
    static constexpr int kind = word_kind<W, M>::value;
    using key_type = Key;
    using value_type = Value;
    using hasher = Hash;
    using iterator = custom_iterator<Key, T, Value>;
    using const_iterator = iterator;
    using ref_type = sg::unordered_ref<kind, word_hash<Key, Hash>>;

    static Derived
    createDeviceObject(const index_t& capacity)
    {
        return createDeviceObject(execution::device, capacity);
    }

    static Derived
    createDeviceObject(execution::device_policy policy, const index_t& capacity)
    {
        Derived d;
        gb300_check(sg_unordered_create_hashed(kind, capacity, policy.stream, &d._handle), "createDeviceObject");
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
        const sg_status st = sg_unordered_create_with_allocator(kind, capacity, 1, &alloc, policy.stream, &d._handle);
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

    // insert(begin, end) over value_type elements (device memory): unordered_base_detail.cuh:996-1017
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
        const std::size_t wb = align256(sizeof(W) * n);
        const std::size_t mb = std::is_same<T, void>::value ? 0 : align256(sizeof(std::uint64_t) * n);
        table_scratch s(_handle, wb + mb + sizeof(std::uint64_t) * n, policy.stream);
        char* base = static_cast<char*>(s.p);
        auto* words = reinterpret_cast<W*>(base);
        auto* mapped = reinterpret_cast<M*>(base + wb);
        auto* hashes = reinterpret_cast<std::uint64_t*>(base + wb + mb);
        k_prepare<Key, T, Hash, value_type><<<grid_of(n), 256, 0, policy.stream>>>(begin, n, words, mapped, hashes);
        gb300_check(cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA, "insert");
        gb300_check(sg_unordered_insert_hashed(_handle, words, std::is_same<T, void>::value ? nullptr : mapped, hashes,
                                               n, nullptr, policy.stream),
                    "insert");
    }

    // erase(begin, end) over keys (device memory): unordered_base_detail.cuh:1045-1066
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
        const std::size_t wb = align256(sizeof(W) * n);
        table_scratch s(_handle, wb + sizeof(std::uint64_t) * n, policy.stream);
        auto* words = reinterpret_cast<W*>(s.p);
        auto* hashes = reinterpret_cast<std::uint64_t*>(static_cast<char*>(s.p) + wb);
        k_prepare_keys<Key, Hash><<<grid_of(n), 256, 0, policy.stream>>>(begin, n, words, hashes, false);
        gb300_check(cudaGetLastError() == cudaSuccess ? SG_OK : SG_ERR_CUDA, "erase");
        gb300_check(sg_unordered_erase_hashed(_handle, words, hashes, n, nullptr, policy.stream), "erase");
    }

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

    // valid(): the library's structural checks plus reachability -- every stored key is found again through
    // the hash of its Key.
    bool
    valid(execution::device_policy policy = execution::device) const
    {
        if (_handle == nullptr)
        {
            return true;
        }
        int32_t ok = 0;
        gb300_check(sg_unordered_valid(_handle, policy.stream, &ok), "valid");
        if (ok == 0)
        {
            return false;
        }
        const std::int64_t cap = _view.total_count + 2;
        const std::size_t wb = align256(sizeof(W) * cap);
        const std::size_t hb = align256(sizeof(std::uint64_t) * cap);
        table_scratch s(_handle, wb + hb + align256(cap) + 256, policy.stream);
        char* base = static_cast<char*>(s.p);
        auto* words = reinterpret_cast<W*>(base);
        auto* hashes = reinterpret_cast<std::uint64_t*>(base + wb);
        auto* flags = reinterpret_cast<std::uint8_t*>(base + wb + hb);
        auto* missing = reinterpret_cast<unsigned int*>(base + wb + hb + align256(cap));
        int64_t n = 0;
        gb300_check(sg_unordered_range_copy(_handle, words, nullptr, policy.stream, &n), "valid");
        if (n == 0)
        {
            return true;
        }
        k_prepare_keys<Key, Hash><<<grid_of(n), 256, 0, policy.stream>>>(nullptr, n, words, hashes, true);
        gb300_check(sg_unordered_contains_hashed(_handle, words, hashes, n, flags, policy.stream), "valid");
        cudaMemsetAsync(missing, 0, sizeof(unsigned int), policy.stream);
        k_all_set<><<<grid_of(n), 256, 0, policy.stream>>>(flags, n, missing);
        unsigned int h_missing = 1;
        cudaMemcpyAsync(&h_missing, missing, sizeof(unsigned int), cudaMemcpyDeviceToHost, policy.stream);
        cudaStreamSynchronize(policy.stream);
        return h_missing == 0;
    }

    custom_range<Key, T>
    device_range(execution::device_policy policy = execution::device)
    {
        int64_t n = 0;
        gb300_check(sg_unordered_device_range(_handle, _range, policy.stream, &n), "device_range");
        return custom_range<Key, T>{ _range, static_cast<index_t>(n), static_cast<const char*>(_view.slots),
                                     sg::detail::kind_consts<kind>::slot_bytes, val_offset() };
    }

    // bucket(key): the fibonacci hashing of Hash(key) (unordered_base_detail.cuh:547-564)
    __host__ __device__ index_t
    bucket(const key_type& key) const
    {
        return static_cast<index_t>(
                sg::detail::fibonacci_bucket(static_cast<std::uint64_t>(Hash{}(key)), _view.bucket_bits));
    }

    // ---- device members
    __device__ iterator
    end() const
    {
        return iterator{ static_cast<const char*>(_view.slots) +
                                 static_cast<std::int64_t>(max_size()) * sg::detail::kind_consts<kind>::slot_bytes,
                         sg::detail::kind_consts<kind>::slot_bytes, val_offset() };
    }

    __device__ index_t
    bucket_size(index_t n) const
    {
        return static_cast<index_t>(ref_type{ _view }.bucket_size(n));
    }

    __device__ iterator
    find(const key_type& key) const
    {
        return at(ref_type{ _view }.find_slot(to_word<W>(key)));
    }

    __device__ bool
    contains(const key_type& key) const
    {
        return ref_type{ _view }.contains(to_word<W>(key));
    }

    __device__ index_t
    count(const key_type& key) const
    {
        return contains(key) ? 1 : 0;
    }

    // Heterogeneous lookups (the reference's KeyLike overloads, src/stdgpu/impl/unordered_base.cuh:241-298):
    // a value comparable with Key through operator== whose Hash equals that of the key it matches, with a
    // transparent Hash.
    template <typename KeyLike, typename H = Hash, typename = typename H::is_transparent,
              typename = std::enable_if_t<!std::is_same<KeyLike, Key>::value>>
    __device__ iterator
    find(const KeyLike& k) const
    {
        return at(ref_type{ _view }.find_slot_if(static_cast<std::uint64_t>(Hash{}(k)),
                                                 [&](W w) { return from_word<Key>(w) == k; }));
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

    __device__ index_t
    erase(const key_type& key) const
    {
        return static_cast<index_t>(ref_type{ _view }.erase(to_word<W>(key)));
    }

    __host__ __device__ bool
    is_null() const
    {
        return _view.slots == nullptr;
    }

protected:
    __host__ __device__ static constexpr int
    val_offset()
    {
        return sg::detail::kind_traits<kind>::is_map ? sg::detail::kind_traits<kind>::val_offset : 0;
    }

    __device__ iterator
    at(std::int64_t slot) const
    {
        return slot < 0 ? end()
                        : iterator{ static_cast<const char*>(_view.slots) + slot * sg::detail::kind_consts<kind>::slot_bytes,
                                    sg::detail::kind_consts<kind>::slot_bytes, val_offset() };
    }

    __device__ pair<iterator, bool>
    insert_impl(const key_type& key, typename ref_type::mapped_type mapped) const
    {
        const std::int64_t s = ref_type{ _view }.insert_slot(to_word<W>(key), mapped);
        return s >= 0 ? pair<iterator, bool>(at(s), true) : pair<iterator, bool>(end(), false);
    }

    sg_unordered* _handle = nullptr;
    sg_unordered_view _view{};
    std::int32_t* _range = nullptr;
    sg_allocator _alloc{}; // the object's own allocator (createDeviceObject(capacity, allocator)), or none
};

template <typename Key, typename T, typename Hash, typename Derived>
class custom_map : public custom_unordered<Key, T, Hash, pair<const Key, T>, Derived>
{
    using base = custom_unordered<Key, T, Hash, pair<const Key, T>, Derived>;
    static_assert(sizeof(T) == 4 || sizeof(T) == 8, "a mapped type of 4 or 8 bytes");
    static_assert(std::is_trivially_copyable<T>::value, "a trivially copyable mapped type");

public:
    using mapped_type = T;
    using typename base::iterator;
    using typename base::value_type;
    using base::erase;
    using base::insert;

    __device__ pair<iterator, bool>
    insert(const value_type& value) const
    {
        return this->insert_impl(value.first, to_word<typename base::ref_type::mapped_type>(value.second));
    }

    __device__ pair<iterator, bool>
    emplace(const Key& key, const T& mapped) const
    {
        return this->insert_impl(key, to_word<typename base::ref_type::mapped_type>(mapped));
    }
};

template <typename Key, typename Hash, typename Derived>
class custom_set : public custom_unordered<Key, void, Hash, Key, Derived>
{
    using base = custom_unordered<Key, void, Hash, Key, Derived>;

public:
    using typename base::iterator;
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

#endif

// A user allocator through the C++ API (include/stdgpu_gb300/stdgpu.cuh): the reference's containers take an
// Allocator type and createDeviceObject(capacity, allocator) allocates the table's arrays through it
// (src/stdgpu/impl/unordered_base_detail.cuh:1254-1308).  A counting device allocator is given to an
// unordered_map<uint64_t, uint32_t> (the library's kinds), an unordered_set of a 6-byte key with a user hash
// (the word-keyed path) and an unordered_map of a 12-byte key (the wide tables).  Checked: every device
// block of each object comes from the allocator (its byte count covers the table's storage, the library's
// process-wide allocator holds nothing for them), the tables work, get_allocator() returns the allocator,
// and destroyDeviceObject gives every block back.  Prints one line per check and "ALL PASS" at the end.
#include <cstdint>
#include <cstdio>
#include <random>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <stdgpu_gb300/stdgpu.cuh>

struct alloc_stats
{
    long long live = 0;  // blocks handed out and not returned
    long long bytes = 0; // their bytes
    long long calls = 0; // allocate calls
};

template <typename T>
struct counting_allocator
{
    using value_type = T;
    alloc_stats* st = nullptr;

    counting_allocator() = default; // the containers hold an allocator member
    explicit counting_allocator(alloc_stats* s)
      : st(s)
    {
    }
    template <typename U>
    counting_allocator(const counting_allocator<U>& o)
      : st(o.st)
    {
    }

    T*
    allocate(std::size_t n)
    {
        void* p = nullptr;
        if (cudaMalloc(&p, n * sizeof(T)) != cudaSuccess)
        {
            return nullptr;
        }
        ++st->live;
        ++st->calls;
        st->bytes += static_cast<long long>(n * sizeof(T));
        return static_cast<T*>(p);
    }

    void
    deallocate(T* p, std::size_t n)
    {
        cudaFree(p);
        --st->live;
        st->bytes -= static_cast<long long>(n * sizeof(T));
    }
};

struct vec3i16
{
    std::int16_t x = 0, y = 0, z = 0;
};
__host__ __device__ inline bool
operator==(const vec3i16& a, const vec3i16& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}
struct vec3i32
{
    std::int32_t x = 0, y = 0, z = 0;
};
__host__ __device__ inline bool
operator==(const vec3i32& a, const vec3i32& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}
struct spatial_hash
{
    template <typename V>
    __host__ __device__ std::size_t
    operator()(const V& k) const
    {
        return (static_cast<std::size_t>(k.x) * 73856093U) ^ (static_cast<std::size_t>(k.y) * 19349669U) ^
               (static_cast<std::size_t>(k.z) * 83492791U);
    }
};

using native_t = stdgpu::unordered_map<std::uint64_t, std::uint32_t, stdgpu::hash<std::uint64_t>,
                                       stdgpu::equal_to<std::uint64_t>,
                                       counting_allocator<stdgpu::pair<const std::uint64_t, std::uint32_t>>>;
using custom_t = stdgpu::unordered_set<vec3i16, spatial_hash, stdgpu::equal_to<vec3i16>, counting_allocator<vec3i16>>;
using wide_t = stdgpu::unordered_map<vec3i32, std::uint64_t, spatial_hash, stdgpu::equal_to<vec3i32>,
                                     counting_allocator<stdgpu::pair<const vec3i32, std::uint64_t>>>;

static int failures = 0;

static void
check(bool ok, const char* name)
{
    std::printf("%s %s\n", ok ? "PASS" : "FAIL", name);
    if (!ok)
    {
        ++failures;
    }
}

template <typename T>
static T*
to_device(const std::vector<T>& h)
{
    T* d = nullptr;
    cudaMalloc(&d, sizeof(T) * (h.size() ? h.size() : 1));
    cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
    return d;
}

template <typename T>
static std::vector<T>
to_host(const T* d, size_t n)
{
    std::vector<T> h(n);
    cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost);
    return h;
}

template <typename Table, typename Key>
__global__ void
k_contains(Table t, const Key* keys, int n, std::uint8_t* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        out[i] = t.contains(keys[i]) ? 1 : 0;
    }
}

template <typename Table, typename Key>
static bool
all_found(const Table& t, const std::vector<Key>& keys)
{
    Key* d = to_device(keys);
    std::uint8_t* f = nullptr;
    cudaMalloc(&f, keys.size());
    k_contains<<<(static_cast<int>(keys.size()) + 255) / 256, 256>>>(t, d, static_cast<int>(keys.size()), f);
    std::vector<std::uint8_t> h = to_host(f, keys.size());
    cudaFree(d);
    cudaFree(f);
    for (auto x : h)
    {
        if (x == 0)
        {
            return false;
        }
    }
    return true;
}

int
main()
{
    std::setvbuf(stdout, nullptr, _IOLBF, 0); // each line out before a failure can end the program
    std::mt19937_64 rng(3);
    const long long lib_before = sg_live_device_allocations();

    // ---- the library's kinds
    {
        alloc_stats st;
        counting_allocator<stdgpu::pair<const std::uint64_t, std::uint32_t>> a(&st);
        native_t m = native_t::createDeviceObject(1 << 16, a);
        sg_geometry g{};
        sg_unordered_geometry_for(SG_MAP_U64_U32, 1 << 16, &g);
        check(st.live == 2 && st.bytes >= g.num_groups * 128 && sg_live_device_allocations() == lib_before,
              "native map: the table's block (slots, header, counters, locks) and the range array from the allocator");
        check(m.get_allocator().st == &st, "native map: get_allocator() returns the allocator");
        std::vector<stdgpu::pair<const std::uint64_t, std::uint32_t>> pairs;
        std::vector<std::uint64_t> keys;
        std::unordered_set<std::uint64_t> uniq;
        for (int i = 0; i < 40000; ++i)
        {
            const std::uint64_t k = rng() >> 2;
            pairs.emplace_back(k, static_cast<std::uint32_t>(i));
            keys.push_back(k);
            uniq.insert(k);
        }
        auto* dp = to_device(pairs);
        m.insert(dp, dp + pairs.size());
        check(m.size() == static_cast<stdgpu::index_t>(uniq.size()) && m.valid() && all_found(m, keys),
              "native map: insert, size, valid, contains");
        cudaFree(dp);
        native_t::destroyDeviceObject(m);
        check(st.live == 0 && st.bytes == 0, "native map: destroyDeviceObject returns every block");
    }

    // ---- the word-keyed path
    {
        alloc_stats st;
        custom_t s = custom_t::createDeviceObject(1 << 14, counting_allocator<vec3i16>(&st));
        check(st.live == 2 && sg_live_device_allocations() == lib_before,
              "custom-key set: the table's block and the range array from the allocator");
        std::vector<vec3i16> keys;
        for (int i = 0; i < 5000; ++i)
        {
            keys.push_back(vec3i16{ static_cast<std::int16_t>(rng() % 200), static_cast<std::int16_t>(rng() % 200),
                                    static_cast<std::int16_t>(rng() % 200) });
        }
        vec3i16* dk = to_device(keys);
        s.insert(dk, dk + keys.size());
        check(s.valid() && all_found(s, keys), "custom-key set: insert, valid, contains");
        cudaFree(dk);
        custom_t::destroyDeviceObject(s);
        check(st.live == 0 && st.bytes == 0, "custom-key set: destroyDeviceObject returns every block");
    }

    // ---- the wide tables
    {
        alloc_stats st;
        counting_allocator<stdgpu::pair<const vec3i32, std::uint64_t>> a(&st);
        wide_t m = wide_t::createDeviceObject(1 << 14, a);
        check(st.live >= 4 && sg_live_device_allocations() == lib_before,
              "wide map: keys, values, header and range array from the allocator");
        std::vector<stdgpu::pair<const vec3i32, std::uint64_t>> pairs;
        std::vector<vec3i32> keys;
        for (int i = 0; i < 6000; ++i)
        {
            const vec3i32 k{ static_cast<std::int32_t>(rng() % 1000), static_cast<std::int32_t>(rng() % 1000),
                             static_cast<std::int32_t>(rng() % 1000) };
            pairs.emplace_back(k, static_cast<std::uint64_t>(i));
            keys.push_back(k);
        }
        auto* dp = to_device(pairs);
        m.insert(dp, dp + pairs.size());
        check(m.valid() && all_found(m, keys), "wide map: insert, valid, contains");
        cudaFree(dp);
        wide_t::destroyDeviceObject(m);
        check(st.live == 0 && st.bytes == 0, "wide map: destroyDeviceObject returns every block");
    }

    // ---- vector and deque
    {
        alloc_stats st;
        using vec_t = stdgpu::vector<std::uint32_t, counting_allocator<std::uint32_t>>;
        vec_t v = vec_t::createDeviceObject(1 << 16, counting_allocator<std::uint32_t>(&st));
        check(st.live >= 4 && st.bytes >= (1 << 16) * 4 && sg_live_device_allocations() == lib_before,
              "vector: data, size and per-slot words from the allocator");
        std::vector<std::uint32_t> h(5000);
        for (int i = 0; i < 5000; ++i)
        {
            h[i] = static_cast<std::uint32_t>(i * 3);
        }
        std::uint32_t* dh = to_device(h);
        v.insert(v.device_end(), dh, dh + h.size());
        check(v.size() == 5000 && v.valid(), "vector: insert at the end, size, valid");
        cudaFree(dh);
        vec_t::destroyDeviceObject(v);
        check(st.live == 0 && st.bytes == 0, "vector: destroyDeviceObject returns every block");
    }
    {
        alloc_stats st;
        using deq_t = stdgpu::deque<std::uint64_t, counting_allocator<std::uint64_t>>;
        deq_t d = deq_t::createDeviceObject(1 << 14, counting_allocator<std::uint64_t>(&st));
        check(st.live >= 5 && sg_live_device_allocations() == lib_before,
              "deque: ring, turn words, counters and per-slot words from the allocator");
        const long long before_range = st.live;
        auto r = d.device_range();
        check(r.size() == 0 && st.live == before_range + 1, "deque: the device_range() array from the allocator too");
        deq_t::destroyDeviceObject(d);
        check(st.live == 0 && st.bytes == 0, "deque: destroyDeviceObject returns every block");
    }

    check(sg_live_device_allocations() == lib_before, "the library's own allocator held nothing for these objects");
    if (cudaDeviceSynchronize() != cudaSuccess)
    {
        std::printf("FAIL cuda error\n");
        return 1;
    }
    std::printf(failures == 0 ? "ALL PASS\n" : "SOME FAILED\n");
    return failures == 0 ? 0 : 1;
}

// Custom key types with a user hash through the C++ API (include/stdgpu_gb300/stdgpu.cuh): a 3 x int16 block
// coordinate with the spatial hash (the key / hash pair of the reference's own tests,
// tests/stdgpu/unordered_map.inc:178-206), the README's block-set and neighbour-update pattern inside a user
// kernel, heterogeneous lookup with a 3 x int32 coordinate, find()->second, bulk erase, bucket(), valid()
// and device_range().  Every result is checked against std::unordered_set / std::unordered_map on the host.
// Prints one line per check and "ALL PASS" at the end.
#include <cstdint>
#include <cstdio>
#include <random>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <stdgpu_gb300/stdgpu.cuh>

struct vec3i16
{
    std::int16_t x = 0, y = 0, z = 0;
    vec3i16() = default;
    __host__ __device__ vec3i16(int a, int b, int c)
      : x(static_cast<std::int16_t>(a))
      , y(static_cast<std::int16_t>(b))
      , z(static_cast<std::int16_t>(c))
    {
    }
};

struct vec3i32
{
    std::int32_t x = 0, y = 0, z = 0;
};

__host__ __device__ inline bool
operator==(const vec3i16& a, const vec3i16& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}

__host__ __device__ inline bool
operator==(const vec3i16& a, const vec3i32& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}

// spatial hash of Teschner et al. (2003); transparent, so a vec3i32 equal to a stored vec3i16 finds it
struct spatial_hash
{
    using is_transparent = void;
    __host__ __device__ std::size_t
    operator()(const vec3i16& k) const
    {
        return (static_cast<std::size_t>(k.x) * 73856093U) ^ (static_cast<std::size_t>(k.y) * 19349669U) ^
               (static_cast<std::size_t>(k.z) * 83492791U);
    }
    __host__ __device__ std::size_t
    operator()(const vec3i32& k) const
    {
        return (static_cast<std::size_t>(k.x) * 73856093U) ^ (static_cast<std::size_t>(k.y) * 19349669U) ^
               (static_cast<std::size_t>(k.z) * 83492791U);
    }
};

struct host_hash
{
    std::size_t
    operator()(const vec3i16& k) const
    {
        return spatial_hash{}(k);
    }
};

using block_set = stdgpu::unordered_set<vec3i16, spatial_hash>;
using block_map = stdgpu::unordered_map<vec3i16, float*, spatial_hash>;
using count_map = stdgpu::unordered_map<vec3i16, std::uint32_t, spatial_hash>;

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

// The README's update pattern: for every block, its 8 lower neighbours that exist in the map enter the set.
__global__ void
compute_update_set(const vec3i16* blocks, int n, block_map map, block_set update_set)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
    {
        return;
    }
    const vec3i16 b = blocks[i];
    for (int j = 0; j < 8; ++j)
    {
        const vec3i16 nb(b.x - (j & 1), b.y - ((j >> 1) & 1), b.z - ((j >> 2) & 1));
        if (map.contains(nb))
        {
            update_set.insert(nb);
        }
    }
}

__global__ void
lookup(const vec3i16* q, int n, block_map map, block_set set, std::uint8_t* in_set, float** ptr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
    {
        return;
    }
    in_set[i] = set.contains(q[i]) ? 1 : 0;
    auto it = map.find(q[i]);
    ptr[i] = it != map.end() ? it->second : nullptr;
}

__global__ void
lookup_wide(const vec3i32* q, int n, block_set set, std::uint8_t* found)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        found[i] = set.contains(q[i]) ? 1 : 0;
    }
}

__global__ void
count_and_erase(const vec3i16* keys, int n, count_map counts, block_set set, int* emplaced, int* erased)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
    {
        return;
    }
    if (counts.emplace(keys[i], static_cast<std::uint32_t>(i)).second)
    {
        atomicAdd(emplaced, 1);
    }
    if (set.erase(keys[i]) == 1)
    {
        atomicAdd(erased, 1);
    }
}

__global__ void
range_keys(stdgpu::detail::custom_range<vec3i16, void> r, vec3i16* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < r.size())
    {
        out[i] = r.key(i);
    }
}

int
main()
{
    std::setvbuf(stdout, nullptr, _IOLBF, 0); // each line out before a failure can end the program
    std::mt19937 rng(7);
    std::uniform_int_distribution<int> coord(-60, 60);
    const int n = 200000;
    std::vector<vec3i16> blocks(n);
    for (auto& b : blocks)
    {
        b = vec3i16(coord(rng), coord(rng), coord(rng));
    }
    std::unordered_set<vec3i16, host_hash> h_blocks(blocks.begin(), blocks.end());

    // bulk insert into a set and a map (the map stores a pointer per block)
    block_set set = block_set::createDeviceObject(1 << 20);
    block_map map = block_map::createDeviceObject(1 << 20);
    vec3i16* d_blocks = to_device(blocks);
    set.insert(d_blocks, d_blocks + n);
    std::vector<stdgpu::pair<const vec3i16, float*>> pairs;
    pairs.reserve(n);
    float* base = reinterpret_cast<float*>(std::uintptr_t{ 0x100000 });
    std::unordered_map<vec3i16, float*, host_hash> h_map;
    for (int i = 0; i < n; ++i)
    {
        pairs.emplace_back(blocks[i], base + i);
        h_map.emplace(blocks[i], base + i);
    }
    // duplicates carry different pointers: which one is stored is unspecified, as in the reference
    auto* d_pairs = to_device(pairs);
    map.insert(d_pairs, d_pairs + n);
    check(set.size() == static_cast<stdgpu::index_t>(h_blocks.size()), "set size after bulk insert of custom keys");
    check(map.size() == static_cast<stdgpu::index_t>(h_map.size()), "map size after bulk insert of custom keys");
    check(set.valid() && map.valid(), "valid() with the user hash");

    // bucket(): fibonacci hashing of the user hash
    {
        const vec3i16 k(3, -4, 5);
        const std::uint64_t h = spatial_hash{}(k);
        const int bits = 20;
        const std::uint64_t drop = 64 - bits;
        const std::uint64_t b = ((h ^ (h >> drop)) * 11400714819323198485ull) >> drop;
        check(set.bucket(k) == static_cast<stdgpu::index_t>(b) && set.bucket_count() == (1 << bits),
              "bucket(key) = fibonacci hashing of Hash(key)");
    }

    // lookups from a user kernel: contains on the set, find()->second on the map
    const int nq = 50000;
    std::vector<vec3i16> q(nq);
    for (auto& k : q)
    {
        k = vec3i16(coord(rng), coord(rng), coord(rng));
    }
    vec3i16* d_q = to_device(q);
    std::uint8_t* d_in = nullptr;
    float** d_ptr = nullptr;
    cudaMalloc(&d_in, nq);
    cudaMalloc(&d_ptr, sizeof(float*) * nq);
    lookup<<<(nq + 255) / 256, 256>>>(d_q, nq, map, set, d_in, d_ptr);
    auto in = to_host(d_in, nq);
    auto ptr = to_host(d_ptr, nq);
    bool ok_in = true, ok_ptr = true;
    for (int i = 0; i < nq; ++i)
    {
        const bool present = h_blocks.count(q[i]) != 0;
        ok_in = ok_in && (in[i] == (present ? 1 : 0));
        ok_ptr = ok_ptr && (present ? ptr[i] != nullptr : ptr[i] == nullptr);
    }
    check(ok_in, "device contains(custom key)");
    check(ok_ptr, "device find(custom key)->second");

    // the value found belongs to one of the key's inserted copies
    {
        std::unordered_map<vec3i16, std::unordered_set<float*>, host_hash> all;
        for (int i = 0; i < n; ++i)
        {
            all[blocks[i]].insert(base + i);
        }
        bool ok = true;
        for (int i = 0; i < nq; ++i)
        {
            if (ptr[i] != nullptr)
            {
                ok = ok && all[q[i]].count(ptr[i]) == 1;
            }
        }
        check(ok, "mapped value is an inserted value of that key");
    }

    // heterogeneous lookup with a 3 x int32 key (transparent hash)
    {
        std::vector<vec3i32> w(nq);
        for (int i = 0; i < nq; ++i)
        {
            w[i] = vec3i32{ q[i].x, q[i].y, q[i].z };
        }
        w[0] = vec3i32{ 70000, 0, 0 }; // equal to no int16 key
        vec3i32* d_w = to_device(w);
        std::uint8_t* d_f = nullptr;
        cudaMalloc(&d_f, nq);
        lookup_wide<<<(nq + 255) / 256, 256>>>(d_w, nq, set, d_f);
        auto f = to_host(d_f, nq);
        bool ok = f[0] == 0;
        for (int i = 1; i < nq; ++i)
        {
            ok = ok && f[i] == in[i];
        }
        check(ok, "heterogeneous contains(vec3i32) on a vec3i16 set");
        cudaFree(d_w);
        cudaFree(d_f);
    }

    // the README's neighbour-update pattern
    {
        block_set update = block_set::createDeviceObject(1 << 21);
        compute_update_set<<<(n + 255) / 256, 256>>>(d_blocks, n, map, update);
        std::unordered_set<vec3i16, host_hash> h_update;
        for (const auto& b : blocks)
        {
            for (int j = 0; j < 8; ++j)
            {
                const vec3i16 nb(b.x - (j & 1), b.y - ((j >> 1) & 1), b.z - ((j >> 2) & 1));
                if (h_map.count(nb))
                {
                    h_update.insert(nb);
                }
            }
        }
        check(update.size() == static_cast<stdgpu::index_t>(h_update.size()), "update set size");
        auto r = update.device_range();
        vec3i16* d_keys = nullptr;
        cudaMalloc(&d_keys, sizeof(vec3i16) * (r.size() + 1));
        range_keys<<<(r.size() + 255) / 256, 256>>>(r, d_keys);
        auto keys = to_host(d_keys, r.size());
        bool ok = static_cast<size_t>(r.size()) == h_update.size();
        std::unordered_set<vec3i16, host_hash> seen;
        for (const auto& k : keys)
        {
            ok = ok && h_update.count(k) == 1 && seen.insert(k).second;
        }
        check(ok, "device_range() of the update set equals the host result");
        check(update.valid(), "update set valid()");
        cudaFree(d_keys);
        block_set::destroyDeviceObject(update);
    }

    // device emplace into a map and device erase from the set, then bulk erase
    {
        count_map counts = count_map::createDeviceObject(1 << 20);
        int* d_c = nullptr;
        cudaMalloc(&d_c, 2 * sizeof(int));
        cudaMemset(d_c, 0, 2 * sizeof(int));
        count_and_erase<<<(nq + 255) / 256, 256>>>(d_q, nq, counts, set, d_c, d_c + 1);
        auto c = to_host(d_c, 2);
        std::unordered_set<vec3i16, host_hash> qs(q.begin(), q.end());
        int erasable = 0;
        for (const auto& k : qs)
        {
            erasable += h_blocks.count(k) ? 1 : 0;
        }
        check(c[0] == static_cast<int>(qs.size()) && counts.size() == static_cast<stdgpu::index_t>(qs.size()),
              "device emplace of custom keys: one success per distinct key");
        check(c[1] == erasable && set.size() == static_cast<stdgpu::index_t>(h_blocks.size() - erasable),
              "device erase of custom keys: one success per present key");
        map.erase(d_blocks, d_blocks + n / 2);
        std::unordered_set<vec3i16, host_hash> left;
        for (int i = n / 2; i < n; ++i)
        {
            left.insert(blocks[i]);
        }
        for (int i = 0; i < n / 2; ++i)
        {
            left.erase(blocks[i]);
        }
        check(map.size() == static_cast<stdgpu::index_t>(left.size()) && map.valid(), "bulk erase of custom keys");
        cudaFree(d_c);
        count_map::destroyDeviceObject(counts);
    }

    block_set::destroyDeviceObject(set);
    block_map::destroyDeviceObject(map);
    cudaFree(d_blocks);
    cudaFree(d_pairs);
    cudaFree(d_q);
    cudaFree(d_in);
    cudaFree(d_ptr);
    const cudaError_t e = cudaDeviceSynchronize();
    check(e == cudaSuccess, "no CUDA error");
    if (failures == 0)
    {
        std::printf("ALL PASS\n");
    }
    return failures == 0 ? 0 : 1;
}

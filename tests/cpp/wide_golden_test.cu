// The wide tables of the C++ API (include/stdgpu_gb300/wide_key.cuh) replaying a scenario recorded from the
// reference itself: unordered_set<vec3i32, Hash> or unordered_map<vec3i32, uint64_t, Hash> (a 12-byte key
// with a user-declared destructor, the spatial hash), bulk insert with repeated keys, lookups, bulk erase,
// final contents, bucket(), and per-key outcomes of device inserts and erases.  The fixture arrays are read
// as raw files from the directory given as argv[1] (written by tests/test_cpp_shim_gpu.py from
// tests/golden/table_vec3i32_<kind>.npz).  Prints one line per check and "ALL PASS" at the end.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <fstream>
#include <map>
#include <string>
#include <tuple>
#include <vector>

#include <stdgpu_gb300/stdgpu.cuh>

struct vec3i32
{
    vec3i32() = default;
    __host__ __device__ vec3i32(std::int32_t a, std::int32_t b, std::int32_t c)
      : x(a)
      , y(b)
      , z(c)
    {
    }
    vec3i32(const vec3i32&) = default;
    vec3i32& operator=(const vec3i32&) = default;
    __host__ __device__ ~vec3i32() {}

    std::int32_t x = 0;
    std::int32_t y = 0;
    std::int32_t z = 0;
};

__host__ __device__ inline bool
operator==(const vec3i32& a, const vec3i32& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}

struct vec_hash
{
    __host__ __device__ std::size_t
    operator()(const vec3i32& k) const
    {
        return (static_cast<std::size_t>(k.x) * 73856093U) ^ (static_cast<std::size_t>(k.y) * 19349669U) ^
               (static_cast<std::size_t>(k.z) * 83492791U);
    }
};

using set_t = stdgpu::unordered_set<vec3i32, vec_hash>;
using map_t = stdgpu::unordered_map<vec3i32, std::uint64_t, vec_hash>;

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
static std::vector<T>
read_file(const std::string& path)
{
    std::ifstream f(path, std::ios::binary | std::ios::ate);
    std::vector<T> v;
    if (!f)
    {
        return v;
    }
    const std::streamsize bytes = f.tellg();
    f.seekg(0);
    v.resize(static_cast<size_t>(bytes) / sizeof(T));
    f.read(reinterpret_cast<char*>(v.data()), static_cast<std::streamsize>(v.size() * sizeof(T)));
    return v;
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

static std::tuple<int, int, int>
tie_of(const vec3i32& k)
{
    return std::make_tuple(k.x, k.y, k.z);
}

template <typename Table>
__global__ void
k_find(Table t, const vec3i32* q, int n, std::uint8_t* found, std::uint64_t* vals)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        auto it = t.find(q[i]);
        found[i] = it != t.end() ? 1 : 0;
        if constexpr (!std::is_same<typename Table::value_type, vec3i32>::value)
        {
            vals[i] = it != t.end() ? it->second : 0;
        }
    }
}

template <typename Table>
__global__ void
k_insert_each(Table t, const vec3i32* keys, const std::uint64_t* vals, int n, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        if constexpr (std::is_same<typename Table::value_type, vec3i32>::value)
        {
            ok[i] = t.insert(keys[i]).second ? 1 : 0;
        }
        else
        {
            ok[i] = t.emplace(keys[i], vals[i]).second ? 1 : 0;
        }
    }
}

template <typename Table>
__global__ void
k_erase_each(Table t, const vec3i32* keys, int n, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        ok[i] = t.erase(keys[i]) == 1 ? 1 : 0;
    }
}

template <typename Range>
__global__ void
k_range_keys(Range r, vec3i32* keys)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < r.size())
    {
        keys[i] = r.key(i);
    }
}

template <typename Range>
__global__ void
k_range_pairs(Range r, vec3i32* keys, std::uint64_t* vals)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < r.size())
    {
        keys[i] = r.key(i);
        vals[i] = r.mapped(i);
    }
}

// per distinct key: how many of its copies succeeded
static std::map<std::tuple<int, int, int>, int>
successes(const std::vector<vec3i32>& keys, const std::vector<std::uint8_t>& ok)
{
    std::map<std::tuple<int, int, int>, int> m;
    for (size_t i = 0; i < keys.size(); ++i)
    {
        m[tie_of(keys[i])] += ok[i];
    }
    return m;
}

template <typename Table, bool IS_MAP>
static void
replay(const std::string& dir)
{
    const auto meta = read_file<std::int64_t>(dir + "/meta.bin");
    // capacity, max_size, bucket_count, size_after_insert, size_after_erase
    const auto keys = read_file<vec3i32>(dir + "/keys.bin");
    const auto values = read_file<std::uint64_t>(dir + "/values.bin");
    const auto queries = read_file<vec3i32>(dir + "/queries.bin");
    const auto found_ref = read_file<std::uint8_t>(dir + "/found.bin");
    const auto found_values = read_file<std::uint64_t>(dir + "/found_values.bin");
    const auto erase = read_file<vec3i32>(dir + "/erase.bin");
    const auto final_keys = read_file<vec3i32>(dir + "/final_keys.bin");
    const auto final_values = read_file<std::uint64_t>(dir + "/final_values.bin");
    const auto buckets = read_file<std::int64_t>(dir + "/buckets.bin");
    const auto insert_flags = read_file<std::uint8_t>(dir + "/insert_flags.bin");
    const auto erase_flags = read_file<std::uint8_t>(dir + "/erase_flags.bin");
    if (meta.size() != 5 || keys.empty() || queries.size() != found_ref.size() || erase.size() != erase_flags.size() ||
        keys.size() != insert_flags.size() || (IS_MAP && (values.size() != keys.size())))
    {
        check(false, "fixture files readable");
        return;
    }
    const int n = static_cast<int>(keys.size());
    const int nq = static_cast<int>(queries.size());
    const int ne = static_cast<int>(erase.size());

    Table t = Table::createDeviceObject(static_cast<stdgpu::index_t>(meta[0]));
    check(t.max_size() == meta[1] && t.bucket_count() == meta[2], "geometry equals the reference's");
    bool ok = true;
    for (size_t i = 0; i < buckets.size(); ++i)
    {
        ok = ok && t.bucket(keys[i]) == buckets[i];
    }
    check(ok, "bucket(key) equals the reference's");

    // bulk insert (repeated keys carry equal values, as the fixture's generator makes them)
    vec3i32* d_keys = to_device(keys);
    if constexpr (IS_MAP)
    {
        std::vector<stdgpu::pair<const vec3i32, std::uint64_t>> pairs;
        pairs.reserve(n);
        for (int i = 0; i < n; ++i)
        {
            pairs.emplace_back(keys[i], values[i]);
        }
        auto* d_pairs = to_device(pairs);
        t.insert(d_pairs, d_pairs + n);
        cudaFree(d_pairs);
    }
    else
    {
        t.insert(d_keys, d_keys + n);
    }
    check(t.size() == meta[3] && t.valid(), "size after bulk insert equals the reference's, valid");

    vec3i32* d_q = to_device(queries);
    std::uint8_t* d_found = nullptr;
    std::uint64_t* d_vals = nullptr;
    cudaMalloc(&d_found, nq);
    cudaMalloc(&d_vals, sizeof(std::uint64_t) * nq);
    k_find<<<(nq + 255) / 256, 256>>>(t, d_q, nq, d_found, d_vals);
    const auto found = to_host(d_found, nq);
    check(found == found_ref, "find(): found flags equal the reference's");
    if constexpr (IS_MAP)
    {
        auto v = to_host(d_vals, nq);
        for (int i = 0; i < nq; ++i)
        {
            v[i] = found[i] ? v[i] : 0;
        }
        check(v == found_values, "find()->second equals the reference's");
    }

    vec3i32* d_e = to_device(erase);
    t.erase(d_e, d_e + ne);
    check(t.size() == meta[4] && t.valid(), "size after bulk erase equals the reference's, valid");

    auto r = t.device_range();
    const int m = static_cast<int>(r.size());
    vec3i32* d_rk = nullptr;
    std::uint64_t* d_rv = nullptr;
    cudaMalloc(&d_rk, sizeof(vec3i32) * (m + 1));
    cudaMalloc(&d_rv, sizeof(std::uint64_t) * (m + 1));
    if constexpr (IS_MAP)
    {
        k_range_pairs<<<(m + 255) / 256, 256>>>(r, d_rk, d_rv);
    }
    else
    {
        k_range_keys<<<(m + 255) / 256, 256>>>(r, d_rk);
    }
    const auto rk = to_host(d_rk, m);
    const auto rv = to_host(d_rv, m);
    std::vector<int> order(m);
    for (int i = 0; i < m; ++i)
    {
        order[i] = i;
    }
    std::sort(order.begin(), order.end(), [&](int a, int b) { return tie_of(rk[a]) < tie_of(rk[b]); });
    ok = static_cast<size_t>(m) == final_keys.size();
    for (int i = 0; ok && i < m; ++i)
    {
        ok = rk[order[i]] == final_keys[i] && (!IS_MAP || rv[order[i]] == final_values[i]);
    }
    check(ok, "device_range(): final contents equal the reference's");

    // device inserts and erases, one thread per element: per distinct key, as many successes as the
    // reference's element-by-element run gave
    Table u = Table::createDeviceObject(static_cast<stdgpu::index_t>(meta[0]));
    std::uint64_t* d_v = to_device(IS_MAP ? values : std::vector<std::uint64_t>(n, 0));
    std::uint8_t* d_ok = nullptr;
    cudaMalloc(&d_ok, n > ne ? n : ne);
    k_insert_each<<<(n + 255) / 256, 256>>>(u, d_keys, d_v, n, d_ok);
    check(successes(keys, to_host(d_ok, n)) == successes(keys, insert_flags) && u.size() == meta[3],
          "device insert: per-key successes equal the reference's");
    k_erase_each<<<(ne + 255) / 256, 256>>>(u, d_e, ne, d_ok);
    check(successes(erase, to_host(d_ok, ne)) == successes(erase, erase_flags) && u.size() == meta[4] && u.valid(),
          "device erase: per-key successes equal the reference's");

    Table::destroyDeviceObject(t);
    Table::destroyDeviceObject(u);
    cudaFree(d_keys);
    cudaFree(d_q);
    cudaFree(d_found);
    cudaFree(d_vals);
    cudaFree(d_e);
    cudaFree(d_rk);
    cudaFree(d_rv);
    cudaFree(d_v);
    cudaFree(d_ok);
}

int
main(int argc, char** argv)
{
    if (argc != 3)
    {
        std::printf("usage: wide_golden_test <fixture dir> <set|map>\n");
        return 2;
    }
    const std::string dir = argv[1];
    if (std::string(argv[2]) == "map")
    {
        replay<map_t, true>(dir);
    }
    else
    {
        replay<set_t, false>(dir);
    }
    check(cudaDeviceSynchronize() == cudaSuccess, "no CUDA error");
    if (failures == 0)
    {
        std::printf("ALL PASS\n");
    }
    return failures == 0 ? 0 : 1;
}

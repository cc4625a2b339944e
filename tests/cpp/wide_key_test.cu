// Element types the precompiled kinds cannot hold, through the C++ API (include/stdgpu_gb300/stdgpu.cuh,
// wide path of wide_key.cuh): the reference's nontrivial-type table -- a 3 x int32 key with a user-declared
// destructor and an empty mapped type, tests/stdgpu/unordered_map.inc:132-161, :238-239, and its
// clear_nontrivial scenario, tests/stdgpu/unordered_datastructure.inc:2461-2478 -- plus 16-byte keys that
// use every bit (the two reserved patterns included), 16-byte mapped values, a mapped type whose destructor
// counts its calls, heterogeneous lookup, device insert races, bucket_size(), device_range(), refusal at
// max_size().  Every result is checked against std::unordered_set / std::unordered_map on the host.
// Prints one line per check and "ALL PASS" at the end.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <random>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <stdgpu_gb300/stdgpu.cuh>

struct vec3int32
{
    vec3int32() = default;
    __host__ __device__ vec3int32(std::int32_t a, std::int32_t b, std::int32_t c)
      : x(a)
      , y(b)
      , z(c)
    {
    }
    __host__ __device__ ~vec3int32() {} // nontrivial destructor, as in the reference's test type
    vec3int32(const vec3int32&) = default;
    vec3int32& operator=(const vec3int32&) = default;

    std::int32_t x = 0;
    std::int32_t y = 0;
    std::int32_t z = 0;
};

struct vec3int16
{
    std::int16_t x = 0, y = 0, z = 0;
};

__host__ __device__ inline bool
operator==(const vec3int32& a, const vec3int32& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}

__host__ __device__ inline bool
operator==(const vec3int32& a, const vec3int16& b)
{
    return a.x == b.x && a.y == b.y && a.z == b.z;
}

// spatial hash of Teschner et al. (2003), transparent over the 16-bit coordinate
struct vec_hash
{
    using is_transparent = void;
    __host__ __device__ std::size_t
    operator()(const vec3int32& k) const
    {
        return (static_cast<std::size_t>(k.x) * 73856093U) ^ (static_cast<std::size_t>(k.y) * 19349669U) ^
               (static_cast<std::size_t>(k.z) * 83492791U);
    }
    __host__ __device__ std::size_t
    operator()(const vec3int16& k) const
    {
        return (*this)(vec3int32(k.x, k.y, k.z));
    }
};

struct host_vec_hash
{
    std::size_t
    operator()(const vec3int32& k) const
    {
        return vec_hash{}(k);
    }
};

struct dummy
{
};

// a 16-byte key with every bit in use (so the two reserved word patterns are ordinary keys)
struct key128
{
    std::uint64_t lo = 0, hi = 0;
};

__host__ __device__ inline bool
operator==(const key128& a, const key128& b)
{
    return a.lo == b.lo && a.hi == b.hi;
}

struct key128_hash
{
    __host__ __device__ std::size_t
    operator()(const key128& k) const
    {
        std::uint64_t h = k.lo * 0x9E3779B97F4A7C15ull ^ (k.hi + 0x632BE59BD9B4E019ull);
        h ^= h >> 29;
        return static_cast<std::size_t>(h * 0xBF58476D1CE4E5B9ull);
    }
};

struct host_key128_hash
{
    std::size_t
    operator()(const key128& k) const
    {
        return key128_hash{}(k);
    }
};

struct alignas(16) payload
{
    float a = 0, b = 0, c = 0, d = 0;
};

__device__ unsigned long long g_destroyed = 0;

// a mapped type whose destructor counts its device calls
struct counted
{
    std::uint32_t v = 0;
    counted() = default;
    __host__ __device__ explicit counted(std::uint32_t x)
      : v(x)
    {
    }
    __host__ __device__ counted(const counted& o)
      : v(o.v)
    {
    }
    __host__ __device__ ~counted()
    {
#if defined(__CUDA_ARCH__)
        atomicAdd(&g_destroyed, 1ull);
#endif
    }
};

using nontrivial_set = stdgpu::unordered_set<vec3int32, vec_hash>;
using nontrivial_map = stdgpu::unordered_map<vec3int32, dummy, vec_hash>;
using wide_payload_map = stdgpu::unordered_map<key128, payload, key128_hash>;
using u64_payload_map = stdgpu::unordered_map<std::uint64_t, payload>;
using counted_map = stdgpu::unordered_map<std::uint32_t, counted>;

static_assert(std::is_base_of<stdgpu::detail::wide_set<vec3int32, vec_hash, nontrivial_set, stdgpu::equal_to<vec3int32>>,
                              nontrivial_set>::value,
              "a 12-byte key that is not trivially copyable takes the wide path and compares with its operator==");
static_assert(std::is_base_of<stdgpu::detail::wide_map<std::uint64_t, payload, stdgpu::hash<std::uint64_t>,
                                                       u64_payload_map>,
                              u64_payload_map>::value,
              "a 16-byte mapped type takes the wide path");

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

static std::uint64_t
fib_bucket(std::uint64_t h, int bits)
{
    const std::uint64_t drop = 64 - bits;
    return ((h ^ (h >> drop)) * 11400714819323198485ull) >> drop;
}

template <typename Table, typename Key>
__global__ void
k_insert_keys(Table t, const Key* keys, int n, int* inserted)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && t.insert(keys[i]).second)
    {
        atomicAdd(inserted, 1);
    }
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
__global__ void
k_erase_keys(Table t, const Key* keys, int n, int* erased)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && t.erase(keys[i]) == 1)
    {
        atomicAdd(erased, 1);
    }
}

__global__ void
k_emplace_dummy(nontrivial_map m, const vec3int32* keys, int n, int* inserted)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && m.emplace(keys[i], dummy{}).second)
    {
        atomicAdd(inserted, 1);
    }
}

template <typename Map, typename Key>
__global__ void
k_find_payload(Map m, const Key* keys, int n, payload* out, std::uint8_t* found)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        auto it = m.find(keys[i]);
        found[i] = it != m.end() ? 1 : 0;
        out[i] = it != m.end() ? it->second : payload{};
    }
}

template <typename Range, typename Key>
__global__ void
k_range_keys(Range r, Key* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < r.size())
    {
        out[i] = r.key(i);
    }
}

template <typename Table>
__global__ void
k_bucket_sizes(Table t, int buckets, unsigned long long* total)
{
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < buckets)
    {
        atomicAdd(total, static_cast<unsigned long long>(t.bucket_size(b)));
    }
}

__global__ void
k_like(nontrivial_set s, const vec3int16* q, int n, std::uint8_t* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        out[i] = s.contains(q[i]) ? 1 : 0;
    }
}

static vec3int32
rand_vec(std::mt19937& rng, int range)
{
    std::uniform_int_distribution<int> c(-range, range);
    return vec3int32(c(rng), c(rng), c(rng));
}

// The reference's clear_nontrivial: one key inserted, size 1, valid; clear; size 0, valid.
static void
clear_nontrivial()
{
    nontrivial_map m = nontrivial_map::createDeviceObject(10000);
    std::vector<vec3int32> k{ vec3int32(-7, -3, 15) };
    vec3int32* d_k = to_device(k);
    int* d_n = nullptr;
    cudaMalloc(&d_n, sizeof(int));
    cudaMemset(d_n, 0, sizeof(int));
    k_emplace_dummy<<<1, 32>>>(m, d_k, 1, d_n);
    check(to_host(d_n, 1)[0] == 1 && m.size() == 1 && m.valid(), "clear_nontrivial: inserted, size 1, valid");
    m.clear();
    check(m.size() == 0 && m.valid(), "clear_nontrivial: cleared, size 0, valid");
    cudaMemset(d_n, 0, sizeof(int));
    k_emplace_dummy<<<1, 32>>>(m, d_k, 1, d_n);
    check(to_host(d_n, 1)[0] == 1 && m.size() == 1, "insert after clear");
    nontrivial_map::destroyDeviceObject(m);
    cudaFree(d_k);
    cudaFree(d_n);
}

// 12-byte keys: bulk and device calls, heterogeneous lookup, buckets, range, erase.
static void
set_of_vec3int32()
{
    std::mt19937 rng(11);
    const int n = 200000;
    std::vector<vec3int32> keys(n);
    for (auto& k : keys)
    {
        k = rand_vec(rng, 40); // about 30 % duplicates
    }
    std::unordered_set<vec3int32, host_vec_hash> h(keys.begin(), keys.end());
    nontrivial_set s = nontrivial_set::createDeviceObject(1 << 19);
    vec3int32* d_keys = to_device(keys);
    s.insert(d_keys, d_keys + n);
    check(s.size() == static_cast<stdgpu::index_t>(h.size()) && s.valid(), "12-byte keys: bulk insert size, valid");

    const vec3int32 probe(3, -4, 5);
    check(s.bucket(probe) == static_cast<stdgpu::index_t>(fib_bucket(vec_hash{}(probe), 19)) &&
                  s.bucket_count() == (1 << 19),
          "bucket(key) = fibonacci hashing of Hash(key)");

    const int nq = 100000;
    std::vector<vec3int32> q(nq);
    std::vector<vec3int16> q16(nq);
    for (int i = 0; i < nq; ++i)
    {
        q[i] = i % 2 == 0 ? keys[rng() % n] : rand_vec(rng, 60);
        q16[i] = vec3int16{ static_cast<std::int16_t>(q[i].x), static_cast<std::int16_t>(q[i].y),
                            static_cast<std::int16_t>(q[i].z) };
    }
    vec3int32* d_q = to_device(q);
    vec3int16* d_q16 = to_device(q16);
    std::uint8_t* d_f = nullptr;
    cudaMalloc(&d_f, nq);
    k_contains<<<(nq + 255) / 256, 256>>>(s, d_q, nq, d_f);
    auto f = to_host(d_f, nq);
    k_like<<<(nq + 255) / 256, 256>>>(s, d_q16, nq, d_f);
    auto f16 = to_host(d_f, nq);
    bool ok = true, ok16 = true;
    for (int i = 0; i < nq; ++i)
    {
        ok = ok && f[i] == (h.count(q[i]) ? 1 : 0);
        ok16 = ok16 && f16[i] == f[i];
    }
    check(ok, "12-byte keys: device contains");
    check(ok16, "12-byte keys: heterogeneous contains(3 x int16)");

    unsigned long long* d_total = nullptr;
    cudaMalloc(&d_total, sizeof(unsigned long long));
    cudaMemset(d_total, 0, sizeof(unsigned long long));
    k_bucket_sizes<<<((1 << 19) + 255) / 256, 256>>>(s, 1 << 19, d_total);
    check(to_host(d_total, 1)[0] == h.size(), "sum of bucket_size() over all buckets = size()");

    // bulk erase of every other distinct key (with repeats in the erase list)
    std::vector<vec3int32> distinct(h.begin(), h.end());
    std::vector<vec3int32> er;
    for (size_t i = 0; i < distinct.size(); i += 2)
    {
        er.push_back(distinct[i]);
        if (i % 6 == 0)
        {
            er.push_back(distinct[i]);
        }
        h.erase(distinct[i]);
    }
    vec3int32* d_er = to_device(er);
    s.erase(d_er, d_er + er.size());
    check(s.size() == static_cast<stdgpu::index_t>(h.size()) && s.valid(), "12-byte keys: bulk erase size, valid");
    k_contains<<<(nq + 255) / 256, 256>>>(s, d_q, nq, d_f);
    f = to_host(d_f, nq);
    ok = true;
    for (int i = 0; i < nq; ++i)
    {
        ok = ok && f[i] == (h.count(q[i]) ? 1 : 0);
    }
    check(ok, "12-byte keys: contains after erase");

    auto r = s.device_range();
    vec3int32* d_out = nullptr;
    cudaMalloc(&d_out, sizeof(vec3int32) * (r.size() + 1));
    k_range_keys<<<(r.size() + 255) / 256, 256>>>(r, d_out);
    auto out = to_host(d_out, r.size());
    ok = static_cast<size_t>(r.size()) == h.size();
    std::unordered_set<vec3int32, host_vec_hash> seen;
    for (const auto& k : out)
    {
        ok = ok && h.count(k) == 1 && seen.insert(k).second;
    }
    check(ok, "12-byte keys: device_range() equals the host set");

    // device inserts racing on duplicates (fresh keys, each 4 times), then device erases racing the same way
    std::vector<vec3int32> fresh;
    std::unordered_set<vec3int32, host_vec_hash> hf;
    while (hf.size() < 20000)
    {
        const vec3int32 k = rand_vec(rng, 1000);
        if (h.count(k) == 0 && hf.insert(k).second)
        {
            for (int c = 0; c < 4; ++c)
            {
                fresh.push_back(k);
            }
        }
    }
    std::shuffle(fresh.begin(), fresh.end(), rng);
    vec3int32* d_fresh = to_device(fresh);
    int* d_n = nullptr;
    cudaMalloc(&d_n, sizeof(int));
    cudaMemset(d_n, 0, sizeof(int));
    const int nf = static_cast<int>(fresh.size());
    k_insert_keys<<<(nf + 255) / 256, 256>>>(s, d_fresh, nf, d_n);
    check(to_host(d_n, 1)[0] == static_cast<int>(hf.size()) &&
                  s.size() == static_cast<stdgpu::index_t>(h.size() + hf.size()) && s.valid(),
          "device insert: exactly one success per distinct key");
    cudaMemset(d_n, 0, sizeof(int));
    k_erase_keys<<<(nf + 255) / 256, 256>>>(s, d_fresh, nf, d_n);
    check(to_host(d_n, 1)[0] == static_cast<int>(hf.size()) && s.size() == static_cast<stdgpu::index_t>(h.size()) &&
                  s.valid(),
          "device erase: exactly one success per distinct key");

    nontrivial_set::destroyDeviceObject(s);
    cudaFree(d_keys);
    cudaFree(d_q);
    cudaFree(d_q16);
    cudaFree(d_f);
    cudaFree(d_total);
    cudaFree(d_er);
    cudaFree(d_out);
    cudaFree(d_fresh);
    cudaFree(d_n);
}

static payload
payload_of(std::uint64_t lo, std::uint64_t hi)
{
    payload p;
    p.a = static_cast<float>(lo & 0xffff);
    p.b = static_cast<float>((lo >> 16) & 0xffff);
    p.c = static_cast<float>(hi & 0xffff);
    p.d = static_cast<float>((hi >> 48) & 0xffff);
    return p;
}

static bool
same(const payload& x, const payload& y)
{
    return x.a == y.a && x.b == y.b && x.c == y.c && x.d == y.d;
}

// 16-byte keys using every bit, the two reserved patterns among them, with 16-byte mapped values.
static void
map_of_key128()
{
    std::mt19937_64 rng(5);
    const int n = 100000;
    std::vector<key128> keys(n);
    for (int i = 0; i < n; ++i)
    {
        keys[i] = i % 5 == 4 ? keys[rng() % i] : key128{ rng(), rng() };
    }
    keys[10] = key128{ ~0ull, ~0ull };     // the never-used pattern
    keys[20] = key128{ ~0ull - 1, ~0ull }; // the erased pattern
    keys[30] = key128{ ~0ull, ~0ull };     // and a repeat of it
    std::vector<stdgpu::pair<const key128, payload>> pairs;
    std::unordered_map<key128, payload, host_key128_hash> h;
    for (const auto& k : keys)
    {
        pairs.emplace_back(k, payload_of(k.lo, k.hi));
        h.emplace(k, payload_of(k.lo, k.hi));
    }
    wide_payload_map m = wide_payload_map::createDeviceObject(1 << 18);
    auto* d_pairs = to_device(pairs);
    m.insert(d_pairs, d_pairs + n);
    check(m.size() == static_cast<stdgpu::index_t>(h.size()) && m.valid(), "16-byte keys: bulk insert size, valid");

    std::vector<key128> q(keys.begin(), keys.begin() + 50000);
    for (int i = 0; i < 20000; ++i)
    {
        q.push_back(key128{ rng(), rng() });
    }
    q.push_back(key128{ ~0ull - 1, ~0ull - 1 });
    const int nq = static_cast<int>(q.size());
    key128* d_q = to_device(q);
    payload* d_v = nullptr;
    std::uint8_t* d_f = nullptr;
    cudaMalloc(&d_v, sizeof(payload) * nq);
    cudaMalloc(&d_f, nq);
    k_find_payload<<<(nq + 255) / 256, 256>>>(m, d_q, nq, d_v, d_f);
    auto v = to_host(d_v, nq);
    auto f = to_host(d_f, nq);
    bool ok = true;
    for (int i = 0; i < nq; ++i)
    {
        const auto it = h.find(q[i]);
        ok = ok && f[i] == (it != h.end() ? 1 : 0) && (it == h.end() || same(v[i], it->second));
    }
    check(ok, "16-byte keys: find()->second, reserved patterns included");

    std::vector<key128> er{ key128{ ~0ull, ~0ull }, key128{ ~0ull - 1, ~0ull }, keys[1], keys[2], keys[2] };
    for (const auto& k : er)
    {
        h.erase(k);
    }
    key128* d_er = to_device(er);
    m.erase(d_er, d_er + er.size());
    check(m.size() == static_cast<stdgpu::index_t>(h.size()) && m.valid(), "16-byte keys: erase of reserved patterns");
    k_find_payload<<<(nq + 255) / 256, 256>>>(m, d_q, nq, d_v, d_f);
    f = to_host(d_f, nq);
    ok = true;
    for (int i = 0; i < nq; ++i)
    {
        ok = ok && f[i] == (h.count(q[i]) ? 1 : 0);
    }
    check(ok, "16-byte keys: find after erase");
    wide_payload_map::destroyDeviceObject(m);
    cudaFree(d_pairs);
    cudaFree(d_q);
    cudaFree(d_v);
    cudaFree(d_f);
    cudaFree(d_er);
}

// Integer keys with the default hash and a 16-byte mapped type; keys all-ones and all-ones minus one included.
static void
u64_keys_with_payload()
{
    std::mt19937_64 rng(9);
    const int n = 60000;
    std::vector<stdgpu::pair<const std::uint64_t, payload>> pairs;
    std::unordered_map<std::uint64_t, payload> h;
    for (int i = 0; i < n; ++i)
    {
        const std::uint64_t k = i == 7 ? ~0ull : (i == 8 ? ~0ull - 1 : rng() >> (i % 3 == 0 ? 44 : 0));
        pairs.emplace_back(k, payload_of(k, k * 3));
        h.emplace(k, payload_of(k, k * 3));
    }
    u64_payload_map m = u64_payload_map::createDeviceObject(1 << 17);
    auto* d_pairs = to_device(pairs);
    m.insert(d_pairs, d_pairs + n);
    std::vector<std::uint64_t> q;
    for (int i = 0; i < n; i += 2)
    {
        q.push_back(pairs[i].first);
        q.push_back(rng());
    }
    const int nq = static_cast<int>(q.size());
    std::uint64_t* d_q = to_device(q);
    payload* d_v = nullptr;
    std::uint8_t* d_f = nullptr;
    cudaMalloc(&d_v, sizeof(payload) * nq);
    cudaMalloc(&d_f, nq);
    k_find_payload<<<(nq + 255) / 256, 256>>>(m, d_q, nq, d_v, d_f);
    auto v = to_host(d_v, nq);
    auto f = to_host(d_f, nq);
    bool ok = m.size() == static_cast<stdgpu::index_t>(h.size()) && m.valid();
    for (int i = 0; i < nq; ++i)
    {
        const auto it = h.find(q[i]);
        ok = ok && f[i] == (it != h.end() ? 1 : 0) && (it == h.end() || same(v[i], it->second));
    }
    check(ok, "u64 keys, 16-byte mapped values: size, valid, find()->second");
    u64_payload_map::destroyDeviceObject(m);
    cudaFree(d_pairs);
    cudaFree(d_q);
    cudaFree(d_v);
    cudaFree(d_f);
}

static unsigned long long
destroyed()
{
    unsigned long long x = 0;
    cudaMemcpyFromSymbol(&x, g_destroyed, sizeof(x));
    return x;
}

// A mapped type with a destructor: erase and clear destroy exactly the stored objects.
static void
mapped_destructors()
{
    const int n = 50000;
    std::vector<stdgpu::pair<const std::uint32_t, counted>> pairs;
    for (int i = 0; i < n; ++i)
    {
        pairs.emplace_back(static_cast<std::uint32_t>(i * 7919u), counted(static_cast<std::uint32_t>(i)));
    }
    for (int i = 0; i < n; i += 10)
    {
        pairs.emplace_back(static_cast<std::uint32_t>(i * 7919u), counted(0)); // repeats: not stored
    }
    const unsigned long long zero = 0;
    cudaMemcpyToSymbol(g_destroyed, &zero, sizeof(zero));
    counted_map m = counted_map::createDeviceObject(1 << 17);
    auto* d_pairs = to_device(pairs);
    m.insert(d_pairs, d_pairs + pairs.size());
    cudaDeviceSynchronize();
    check(m.size() == n && destroyed() == 0, "mapped type with a destructor: inserted, nothing destroyed");
    std::vector<std::uint32_t> er;
    for (int i = 0; i < n; i += 4)
    {
        er.push_back(static_cast<std::uint32_t>(i * 7919u));
        er.push_back(static_cast<std::uint32_t>(i * 7919u));
    }
    std::uint32_t* d_er = to_device(er);
    m.erase(d_er, d_er + er.size());
    cudaDeviceSynchronize();
    const unsigned long long ne = er.size() / 2;
    check(m.size() == static_cast<stdgpu::index_t>(n - ne) && destroyed() == ne && m.valid(),
          "erase destroys each erased object once");
    m.clear();
    cudaDeviceSynchronize();
    check(m.size() == 0 && destroyed() == static_cast<unsigned long long>(n) && m.valid(),
          "clear destroys every stored object");
    m.insert(d_pairs, d_pairs + 100);
    counted_map::destroyDeviceObject(m);
    check(destroyed() == static_cast<unsigned long long>(n + 100), "destroyDeviceObject destroys what is stored");
    cudaFree(d_pairs);
    cudaFree(d_er);
}

// Refusal: a full table (size() == max_size()) takes no more keys.
static void
refusal_when_full()
{
    nontrivial_set s = nontrivial_set::createDeviceObject(8);
    std::vector<vec3int32> keys;
    for (int i = 0; i < 1000; ++i)
    {
        keys.push_back(vec3int32(i, -i, 2 * i));
    }
    vec3int32* d_keys = to_device(keys);
    s.insert(d_keys, d_keys + keys.size());
    check(s.size() == s.max_size() && s.full() && s.valid(), "bulk insert fills the table to max_size() and stops");
    int* d_n = nullptr;
    cudaMalloc(&d_n, sizeof(int));
    cudaMemset(d_n, 0, sizeof(int));
    k_insert_keys<<<4, 256>>>(s, d_keys, 1000, d_n);
    check(to_host(d_n, 1)[0] == 0 && s.size() == s.max_size(), "device insert into a full table is refused");
    nontrivial_set::destroyDeviceObject(s);
    cudaFree(d_keys);
    cudaFree(d_n);
}

template <typename Table>
__global__ void
k_churn(Table t, const vec3int32* keys, const std::uint8_t* is_insert, int n, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        ok[i] = is_insert[i] != 0 ? (t.insert(keys[i]).second ? 1 : 0) : (t.erase(keys[i]) == 1 ? 1 : 0);
    }
}

// Device-only insert / erase churn of 12-byte keys (the reference's voxel-block pattern): every launch
// inserts some keys of a small set and erases others, three threads per key, in shuffled thread order.
// After every launch the per-key outcomes and size() equal a std::unordered_set model: erased slots are
// reused, so no insert is refused below max_size().  Then blocks of max_size() keys are inserted and erased
// until no never-used slot is left, and the table still fills to exactly max_size().
static void
device_churn_reuses_erased_slots()
{
    std::mt19937 rng(77);
    nontrivial_set s = nontrivial_set::createDeviceObject(64);
    const int max_size = static_cast<int>(s.max_size());
    std::vector<vec3int32> universe;
    for (int i = 0; i < 40; ++i)
    {
        universe.push_back(vec3int32(i * 7 - 100, i % 5, -i));
    }
    std::unordered_set<int> present;
    bool same = true;
    for (int l = 0; l < 300; ++l)
    {
        std::vector<vec3int32> keys;
        std::vector<std::uint8_t> ins;
        std::vector<int> which;
        for (int k = 0; k < 40; ++k)
        {
            const int r = static_cast<int>(rng() % 3); // 0 nothing, 1 insert, 2 erase
            for (int c = 0; r != 0 && c < 3; ++c)
            {
                keys.push_back(universe[k]);
                ins.push_back(r == 1 ? 1 : 0);
                which.push_back(k);
            }
        }
        std::vector<int> order(keys.size());
        for (size_t i = 0; i < order.size(); ++i)
        {
            order[i] = static_cast<int>(i);
        }
        std::shuffle(order.begin(), order.end(), rng);
        std::vector<vec3int32> k2;
        std::vector<std::uint8_t> i2;
        std::vector<int> w2;
        for (int o : order)
        {
            k2.push_back(keys[o]);
            i2.push_back(ins[o]);
            w2.push_back(which[o]);
        }
        const int n = static_cast<int>(k2.size());
        if (n == 0)
        {
            continue;
        }
        vec3int32* dk = to_device(k2);
        std::uint8_t* di = to_device(i2);
        std::uint8_t* dok = nullptr;
        cudaMalloc(&dok, n);
        k_churn<<<(n + 127) / 128, 128>>>(s, dk, di, n, dok);
        const std::vector<std::uint8_t> ok = to_host(dok, n);
        std::vector<int> wins(40, 0);
        for (int i = 0; i < n; ++i)
        {
            wins[w2[i]] += ok[i];
        }
        for (int k = 0; k < 40; ++k)
        {
            bool inserted = false, erased = false;
            for (int i = 0; i < n; ++i)
            {
                inserted |= w2[i] == k && i2[i] == 1;
                erased |= w2[i] == k && i2[i] == 0;
            }
            if (inserted)
            {
                same = same && wins[k] == (present.count(k) ? 0 : 1);
                present.insert(k);
            }
            else if (erased)
            {
                same = same && wins[k] == (present.count(k) ? 1 : 0);
                present.erase(k);
            }
        }
        same = same && s.size() == static_cast<stdgpu::index_t>(present.size());
        cudaFree(dk);
        cudaFree(di);
        cudaFree(dok);
    }
    check(same && s.valid(), "wide device churn: per-key outcomes and size() equal the model after every launch");
    // clear the rest, then blocks of max_size() keys in and out until every slot has been used
    nontrivial_set::destroyDeviceObject(s);
    s = nontrivial_set::createDeviceObject(64);
    bool filled = true;
    for (int b = 0; b < 4; ++b)
    {
        std::vector<vec3int32> blk;
        std::vector<std::uint8_t> one(max_size, 1), zero(max_size, 0);
        for (int i = 0; i < max_size; ++i)
        {
            blk.push_back(vec3int32(1000 * b + i, b, i));
        }
        vec3int32* dk = to_device(blk);
        std::uint8_t* d1 = to_device(one);
        std::uint8_t* d0 = to_device(zero);
        std::uint8_t* dok = nullptr;
        cudaMalloc(&dok, max_size);
        k_churn<<<(max_size + 127) / 128, 128>>>(s, dk, d1, max_size, dok);
        int c = 0;
        for (auto x : to_host(dok, max_size))
        {
            c += x;
        }
        filled = filled && c == max_size && s.size() == max_size;
        if (b < 3)
        {
            k_churn<<<(max_size + 127) / 128, 128>>>(s, dk, d0, max_size, dok);
            filled = filled && s.size() == 0;
        }
        cudaFree(dk);
        cudaFree(d1);
        cudaFree(d0);
        cudaFree(dok);
    }
    check(filled && s.valid(), "wide device churn: erased slots refill the table to exactly max_size()");
    nontrivial_set::destroyDeviceObject(s);
}

int
main()
{
    std::setvbuf(stdout, nullptr, _IOLBF, 0); // each line out before a failure can end the program
    clear_nontrivial();
    set_of_vec3int32();
    map_of_key128();
    u64_keys_with_payload();
    mapped_destructors();
    refusal_when_full();
    device_churn_reuses_erased_slots();
    const cudaError_t e = cudaDeviceSynchronize();
    check(e == cudaSuccess, "no CUDA error");
    if (failures == 0)
    {
        std::printf("ALL PASS\n");
    }
    return failures == 0 ? 0 : 1;
}

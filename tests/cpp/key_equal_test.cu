// Keys compared by KeyEqual through the C++ API (include/stdgpu_gb300/stdgpu.cuh): the reference compares a
// probed key with every stored candidate through KeyEqual (src/stdgpu/impl/unordered_base_detail.cuh:661,
// :673), so two keys whose bytes differ are one key when KeyEqual says so.  Two cases, each checked against
// std::unordered_set / std::unordered_map with the same Hash and KeyEqual on the host:
//   * a tagged key {x, tag} whose Hash and KeyEqual look at x only: bulk insert of many tags per x, device
//     contains / find with other tags, bulk erase with other tags, device inserts of equal keys racing in
//     one launch, device erase, device_range(), valid();
//   * float keys with the default equal_to<float>, whose bytes do not decide equality (+0.0 == -0.0):
//     bulk and device inserts, find with the other zero, mapped values.
// Prints one line per check and "ALL PASS" at the end.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <random>
#include <type_traits>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <stdgpu_gb300/stdgpu.cuh>

struct tagged
{
    std::int32_t x = 0;
    std::int32_t tag = 0;
};

struct x_hash
{
    __host__ __device__ std::size_t
    operator()(const tagged& k) const
    {
        std::uint64_t h = static_cast<std::uint64_t>(static_cast<std::uint32_t>(k.x)) * 0x9E3779B97F4A7C15ull;
        return static_cast<std::size_t>(h ^ (h >> 31));
    }
};

struct x_equal
{
    __host__ __device__ bool
    operator()(const tagged& a, const tagged& b) const
    {
        return a.x == b.x;
    }
};

// +0.0 and -0.0 hash alike, as equal keys must
struct float_hash
{
    __host__ __device__ std::size_t
    operator()(float f) const
    {
        std::uint32_t b = 0;
        if (f != 0.0F)
        {
            std::memcpy(&b, &f, 4);
        }
        return static_cast<std::size_t>(static_cast<std::uint64_t>(b) * 0xBF58476D1CE4E5B9ull);
    }
};

using tag_set = stdgpu::unordered_set<tagged, x_hash, x_equal>;
using float_map = stdgpu::unordered_map<float, std::uint32_t, float_hash>;
static_assert(std::is_base_of<stdgpu::detail::wide_set<tagged, x_hash, tag_set, x_equal>, tag_set>::value,
              "a user KeyEqual takes the wide tables");
static_assert(std::is_base_of<stdgpu::detail::wide_map<float, std::uint32_t, float_hash, float_map,
                                                       stdgpu::equal_to<float>>,
                              float_map>::value,
              "floating-point keys compare with equal_to<float>");

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
k_insert_keys(Table t, const Key* keys, int n, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        ok[i] = t.insert(keys[i]).second ? 1 : 0;
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
k_erase_keys(Table t, const Key* keys, int n, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        ok[i] = t.erase(keys[i]) == 1 ? 1 : 0;
    }
}

__global__ void
k_find_tags(tag_set s, const tagged* keys, int n, std::int32_t* stored_tag, std::uint8_t* found)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        auto it = s.find(keys[i]);
        found[i] = it != s.end() ? 1 : 0;
        stored_tag[i] = it != s.end() ? (*it).tag : -1;
    }
}

__global__ void
k_find_floats(float_map m, const float* keys, int n, std::uint32_t* vals, std::uint8_t* found)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        auto it = m.find(keys[i]);
        found[i] = it != m.end() ? 1 : 0;
        vals[i] = it != m.end() ? it->second : 0u;
    }
}

__global__ void
k_emplace_floats(float_map m, const float* keys, const std::uint32_t* vals, int n, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        ok[i] = m.emplace(keys[i], vals[i]).second ? 1 : 0;
    }
}

template <typename Range>
__global__ void
k_range_keys(Range r, tagged* out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < r.size())
    {
        out[i] = r.key(i);
    }
}

struct host_x_hash
{
    std::size_t
    operator()(const tagged& k) const
    {
        return x_hash{}(k);
    }
};
struct host_x_equal
{
    bool
    operator()(const tagged& a, const tagged& b) const
    {
        return a.x == b.x;
    }
};
using model_set = std::unordered_set<tagged, host_x_hash, host_x_equal>;

static int
count(const std::vector<std::uint8_t>& v)
{
    int c = 0;
    for (auto x : v)
    {
        c += x;
    }
    return c;
}

int
main()
{
    std::setvbuf(stdout, nullptr, _IOLBF, 0); // each line out before a failure can end the program
    std::mt19937 rng(7);
    constexpr int kBlock = 256;
    auto grid = [](int n) { return (n + kBlock - 1) / kBlock; };

    // ---------------- tagged keys: one key per x, whatever the tag
    {
        const int n = 40000;
        const int xs = 9000;
        tag_set s = tag_set::createDeviceObject(20000);
        model_set model;
        std::vector<tagged> keys(n);
        for (auto& k : keys)
        {
            k.x = static_cast<std::int32_t>(rng() % xs);
            k.tag = static_cast<std::int32_t>(rng() & 0xffff);
            model.insert(k);
        }
        tagged* dk = to_device(keys);
        s.insert(dk, dk + n);
        check(s.size() == static_cast<stdgpu::index_t>(model.size()) && s.valid(),
              "bulk insert: one element per x, whatever the tags");

        // the stored tag of each x is one of the tags inserted for it
        std::vector<tagged> probe(xs + 500);
        for (int i = 0; i < static_cast<int>(probe.size()); ++i)
        {
            probe[i].x = i;
            probe[i].tag = -7; // never inserted
        }
        tagged* dp = to_device(probe);
        std::int32_t* dt = nullptr;
        std::uint8_t* df = nullptr;
        cudaMalloc(&dt, sizeof(std::int32_t) * probe.size());
        cudaMalloc(&df, probe.size());
        k_find_tags<<<grid(static_cast<int>(probe.size())), kBlock>>>(s, dp, static_cast<int>(probe.size()), dt, df);
        std::vector<std::int32_t> tags = to_host(dt, probe.size());
        std::vector<std::uint8_t> found = to_host(df, probe.size());
        bool ok = true;
        for (size_t i = 0; i < probe.size(); ++i)
        {
            const bool want = model.count(probe[i]) != 0;
            ok = ok && (found[i] != 0) == want;
            if (want && found[i] != 0)
            {
                bool tag_ok = false;
                for (const auto& k : keys)
                {
                    tag_ok = tag_ok || (k.x == probe[i].x && k.tag == tags[i]);
                }
                ok = ok && tag_ok;
            }
        }
        check(ok, "device find with another tag: found exactly the inserted x, with one of its own tags");

        // bulk erase of every third x, through keys with fresh tags
        std::vector<tagged> gone;
        for (int x = 0; x < xs; x += 3)
        {
            gone.push_back(tagged{ x, 99999 });
            model.erase(tagged{ x, 0 });
        }
        tagged* dg = to_device(gone);
        s.erase(dg, dg + gone.size());
        check(s.size() == static_cast<stdgpu::index_t>(model.size()) && s.valid(),
              "bulk erase with other tags removes the equal keys");

        // device inserts racing: many equal keys (other tags) in one launch, one success per absent x
        const int m = 30000;
        std::vector<tagged> race(m);
        for (auto& k : race)
        {
            k.x = static_cast<std::int32_t>(rng() % (xs + 3000));
            k.tag = static_cast<std::int32_t>(rng() & 0xffff);
        }
        model_set before = model;
        std::unordered_set<std::int32_t> new_x;
        for (const auto& k : race)
        {
            if (before.count(k) == 0)
            {
                new_x.insert(k.x);
            }
            model.insert(k);
        }
        tagged* dr = to_device(race);
        std::uint8_t* dok = nullptr;
        cudaMalloc(&dok, m);
        k_insert_keys<<<grid(m), kBlock>>>(s, dr, m, dok);
        std::vector<std::uint8_t> ins = to_host(dok, m);
        std::unordered_map<std::int32_t, int> wins;
        for (int i = 0; i < m; ++i)
        {
            wins[race[i].x] += ins[i];
        }
        bool one_each = true;
        for (const auto& w : wins)
        {
            one_each = one_each && w.second == (new_x.count(w.first) != 0 ? 1 : 0);
        }
        check(one_each && count(ins) == static_cast<int>(new_x.size()) &&
                      s.size() == static_cast<stdgpu::index_t>(model.size()) && s.valid(),
              "device inserts of equal keys in one launch: exactly one success per absent x");

        // device erase with other tags, racing on equal keys: one success per present x
        std::vector<tagged> del(m);
        for (auto& k : del)
        {
            k.x = static_cast<std::int32_t>(rng() % (xs + 3000));
            k.tag = -static_cast<std::int32_t>(rng() & 0xffff) - 1;
        }
        std::unordered_set<std::int32_t> present_x;
        for (const auto& k : del)
        {
            if (model.count(k) != 0)
            {
                present_x.insert(k.x);
            }
        }
        for (const auto& k : del)
        {
            model.erase(k);
        }
        tagged* dd = to_device(del);
        k_erase_keys<<<grid(m), kBlock>>>(s, dd, m, dok);
        std::vector<std::uint8_t> er = to_host(dok, m);
        std::unordered_map<std::int32_t, int> erased_x;
        for (int i = 0; i < m; ++i)
        {
            erased_x[del[i].x] += er[i];
        }
        bool erase_once = true;
        for (const auto& e : erased_x)
        {
            erase_once = erase_once && e.second == (present_x.count(e.first) != 0 ? 1 : 0);
        }
        check(erase_once && s.size() == static_cast<stdgpu::index_t>(model.size()) && s.valid(),
              "device erases of equal keys in one launch: exactly one success per present x");

        // device_range(): every x of the model once
        auto r = s.device_range();
        tagged* dout = nullptr;
        cudaMalloc(&dout, sizeof(tagged) * (r.size() > 0 ? r.size() : 1));
        k_range_keys<<<grid(static_cast<int>(r.size())), kBlock>>>(r, dout);
        std::vector<tagged> listed = to_host(dout, static_cast<size_t>(r.size()));
        std::vector<std::int32_t> lx, mx;
        for (const auto& k : listed)
        {
            lx.push_back(k.x);
        }
        for (const auto& k : model)
        {
            mx.push_back(k.x);
        }
        std::sort(lx.begin(), lx.end());
        std::sort(mx.begin(), mx.end());
        check(lx == mx, "device_range(): each x of the model exactly once");

        tag_set::destroyDeviceObject(s);
        for (void* p : { static_cast<void*>(dk), static_cast<void*>(dp), static_cast<void*>(dt),
                         static_cast<void*>(df), static_cast<void*>(dg), static_cast<void*>(dr),
                         static_cast<void*>(dok), static_cast<void*>(dd), static_cast<void*>(dout) })
        {
            cudaFree(p);
        }
    }

    // ---------------- float keys: +0.0 and -0.0 are one key
    {
        float_map m = float_map::createDeviceObject(4096);
        std::vector<float> keys;
        std::vector<std::uint32_t> vals;
        keys.push_back(0.0F);
        vals.push_back(11u);
        keys.push_back(-0.0F);
        vals.push_back(22u);
        std::uniform_real_distribution<float> u(-1000.0F, 1000.0F);
        for (int i = 0; i < 1500; ++i)
        {
            keys.push_back(u(rng));
            vals.push_back(static_cast<std::uint32_t>(1000 + i));
        }
        // bulk insert of the first two (value_type pairs): one element, the first zero's value
        std::vector<stdgpu::pair<const float, std::uint32_t>> first2;
        first2.emplace_back(keys[0], vals[0]);
        first2.emplace_back(keys[1], vals[1]);
        auto* d2 = to_device(first2);
        m.insert(d2, d2 + 2); // +0.0 and -0.0 in one bulk call: one element, either value
        check(m.size() == 1 && m.valid(), "float keys: a bulk insert of +0.0 and -0.0 stores one element");
        float* dk = to_device(keys);
        std::uint32_t* dv = to_device(vals);
        std::uint8_t* dok = nullptr;
        cudaMalloc(&dok, keys.size());
        k_emplace_floats<<<grid(static_cast<int>(keys.size())), kBlock>>>(m, dk, dv, static_cast<int>(keys.size()),
                                                                       dok);
        std::vector<std::uint8_t> ok = to_host(dok, keys.size());
        std::unordered_map<float, std::uint32_t> model; // std::hash<float> and == treat the zeros as one key
        model.emplace(keys[0], vals[0]);
        for (size_t i = 0; i < keys.size(); ++i)
        {
            model.emplace(keys[i], vals[i]);
        }
        check(ok[0] == 0 && ok[1] == 0 && m.size() == static_cast<stdgpu::index_t>(model.size()) && m.valid(),
              "float keys: -0.0 is the key +0.0 already present (device emplace refused for both zeros)");
        std::vector<float> probe = { -0.0F, 0.0F, 1e9F };
        for (size_t i = 2; i < keys.size(); i += 7)
        {
            probe.push_back(keys[i]);
        }
        float* dp = to_device(probe);
        std::uint32_t* dpv = nullptr;
        std::uint8_t* dpf = nullptr;
        cudaMalloc(&dpv, 4 * probe.size());
        cudaMalloc(&dpf, probe.size());
        k_find_floats<<<grid(static_cast<int>(probe.size())), kBlock>>>(m, dp, static_cast<int>(probe.size()), dpv,
                                                                     dpf);
        std::vector<std::uint32_t> got = to_host(dpv, probe.size());
        std::vector<std::uint8_t> fnd = to_host(dpf, probe.size());
        bool all = true;
        for (size_t i = 2; i < probe.size(); ++i)
        {
            auto it = model.find(probe[i]);
            all = all && (fnd[i] != 0) == (it != model.end()) && (it == model.end() || got[i] == it->second);
        }
        check(all && fnd[0] != 0 && fnd[1] != 0 && got[0] == got[1] && (got[0] == 11u || got[0] == 22u),
              "float find: both zeros find the one zero element; the other keys as the model");
        float_map::destroyDeviceObject(m);
        for (void* p : { static_cast<void*>(d2), static_cast<void*>(dk), static_cast<void*>(dv),
                         static_cast<void*>(dok), static_cast<void*>(dp), static_cast<void*>(dpv),
                         static_cast<void*>(dpf) })
        {
            cudaFree(p);
        }
    }

    if (cudaDeviceSynchronize() != cudaSuccess)
    {
        std::printf("FAIL cuda error\n");
        return 1;
    }
    std::printf(failures == 0 ? "ALL PASS\n" : "SOME FAILED\n");
    return failures == 0 ? 0 : 1;
}

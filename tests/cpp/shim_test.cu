// Scenarios of the reference's own unordered / vector tests (tests/stdgpu/unordered_datastructure.inc,
// tests/stdgpu/vector.inc), written against the C++ API of include/stdgpu_gb300/stdgpu.cuh: native
// device calls inside user kernels plus the host bulk calls.  Prints one line per check and ends with
// "ALL PASS" when every check holds.
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <random>
#include <set>
#include <string>
#include <unordered_set>
#include <unordered_map>
#include <vector>

#include <stdgpu_gb300/stdgpu.cuh>

using map_t = stdgpu::unordered_map<std::uint64_t, std::uint32_t>;
using set_t = stdgpu::unordered_set<std::uint64_t>;

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

static void
check(bool ok, const std::string& name)
{
    check(ok, name.c_str());
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

static std::vector<std::uint64_t>
unique_keys(size_t n, std::uint64_t seed)
{
    std::mt19937_64 rng(seed);
    std::unordered_set<std::uint64_t> s;
    std::vector<std::uint64_t> out;
    while (out.size() < n)
    {
        std::uint64_t k = rng() >> 1;
        if (s.insert(k).second)
        {
            out.push_back(k);
        }
    }
    return out;
}

__global__ void
k_insert(map_t m, const std::uint64_t* keys, int n, int* inserted)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        inserted[i] = m.insert(stdgpu::pair<const std::uint64_t, std::uint32_t>(keys[i], static_cast<std::uint32_t>(i))).second;
    }
}

__global__ void
k_emplace(map_t m, const std::uint64_t* keys, int n, int* inserted)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        inserted[i] = m.emplace(keys[i], static_cast<std::uint32_t>(i)).second;
    }
}

__global__ void
k_erase(map_t m, const std::uint64_t* keys, int n, int* erased)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        erased[i] = m.erase(keys[i]);
    }
}

__global__ void
k_insert_and_erase(map_t m, const std::uint64_t* keys, int n, int* inserted, int* erased)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        inserted[i] = m.emplace(keys[i], 1u).second;
        erased[i] = m.erase(keys[i]);
    }
}

__global__ void
k_insert_same(set_t s, std::uint64_t key, int n, int* inserted)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        inserted[i] = s.insert(key).second;
    }
}

__global__ void
k_find_values(map_t m, const std::uint64_t* keys, int n, int* ok)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        auto it = m.find(keys[i]);
        ok[i] = (it != m.end() && it->first == keys[i] && it->second == static_cast<std::uint32_t>(i)) ? 1 : 0;
    }
}

// find from a warp whose lanes call in different shapes: every lane (a full warp, the cooperative read),
// odd lanes only (a partial warp), and full warps in which some lanes hold the out-of-band keys or keys that
// are absent.  want[i]: the expected value + 1, or 0 when absent.
__global__ void
k_find_shapes(map_t m, const std::uint64_t* keys, const std::uint32_t* want, int n, int mode, int* bad)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n || (mode == 1 && (threadIdx.x & 1) == 0))
    {
        return;
    }
    auto it = m.find(keys[i]);
    const std::uint32_t got = it != m.end() ? it->second + 1u : 0u;
    if (got != want[i] || m.contains(keys[i]) != (want[i] != 0u))
    {
        atomicAdd(bad, 1);
    }
}

__global__ void
k_count_sum(map_t m, const std::uint64_t* keys, int n, unsigned long long* sum)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        atomicAdd(sum, static_cast<unsigned long long>(m.count(keys[i])));
    }
}

__global__ void
k_bucket_size_sum(map_t m, unsigned long long* sum)
{
    int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b < m.bucket_count())
    {
        atomicAdd(sum, static_cast<unsigned long long>(m.bucket_size(b)));
    }
}

__global__ void
k_range_sum(stdgpu::device_indexed_range<map_t::value_type> r, unsigned long long* sum)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < r.size())
    {
        atomicAdd(sum, static_cast<unsigned long long>(r[i].second));
    }
}

__global__ void
k_push_if(stdgpu::vector<std::uint32_t> v, int n, int* pushed)
{
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && (i % 3) == 0)
    {
        pushed[i] = v.push_back(static_cast<std::uint32_t>(i));
    }
}

// vector.inc:1022-1056 simultaneous_push_back_and_pop_back: every thread pushes its value, pops one element
// and pushes what it popped into a second vector, all in one launch
__global__ void
vector_push_then_pop(stdgpu::vector<int> pool, stdgpu::vector<int> validation, const int* values, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        pool.push_back(values[i]);
        const auto popped = pool.pop_back();
        if (popped.second)
        {
            validation.push_back(popped.first);
        }
    }
}

// deque.inc:1494-1700 simultaneous_*: every thread pushes its value at one end, pops one element from one
// end and pushes what it popped into a second deque; mode bit 0: push_front (else push_back), bit 1:
// pop_front (else pop_back)
__global__ void
deque_push_then_pop(stdgpu::deque<int> pool, stdgpu::deque<int> validation, const int* values, int n, int mode)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        if (mode & 1)
        {
            pool.push_front(values[i]);
        }
        else
        {
            pool.push_back(values[i]);
        }
        const auto popped = (mode & 2) ? pool.pop_front() : pool.pop_back();
        if (popped.second)
        {
            if (mode & 1)
            {
                validation.push_front(popped.first);
            }
            else
            {
                validation.push_back(popped.first);
            }
        }
    }
}

// one device call per thread: 0 push_back, 1 push_front, 2 emplace_front, 3 pop_back, 4 pop_front
__global__ void
deque_calls(stdgpu::deque<int> d, const int* values, int n, int op, int* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        bool r = false;
        switch (op)
        {
            case 0:
                r = d.push_back(values[i]);
                break;
            case 1:
                r = d.push_front(values[i]);
                break;
            case 2:
                r = d.emplace_front(values[i]);
                break;
            case 3:
                r = d.pop_back().second;
                break;
            default:
                r = d.pop_front().second;
                break;
        }
        ok[i] = r ? 1 : 0;
    }
}

static long long
count_ok(const std::uint8_t* d, int n)
{
    long long c = 0;
    for (auto x : to_host(d, n))
    {
        c += x;
    }
    return c;
}

// deque: thread i pushes values[i] when i is even, else pops the front (deque.inc:406-560 pushes and pops
// from many threads of one launch)
__global__ void
deque_mixed(stdgpu::deque<std::uint64_t> d, const std::uint64_t* values, int n, std::uint64_t* popped,
            std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n)
    {
        return;
    }
    if ((i & 1) == 0)
    {
        ok[i] = d.push_back(values[i]) ? 1 : 0;
    }
    else
    {
        auto r = d.pop_front();
        ok[i] = r.second ? 1 : 0;
        popped[i] = r.second ? r.first : 0;
    }
}

__global__ void
deque_fill(stdgpu::deque<std::uint64_t> d, const std::uint64_t* values, int n, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        ok[i] = d.push_back(values[i]) ? 1 : 0;
    }
}

__global__ void
deque_drain(stdgpu::deque<std::uint64_t> d, int n, std::uint64_t* popped, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        auto r = d.pop_front();
        ok[i] = r.second ? 1 : 0;
        popped[i] = r.second ? r.first : 0;
    }
}

__global__ void
queue_push(stdgpu::queue<std::uint32_t> q, int n, int* pushed)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && q.push(static_cast<std::uint32_t>(i)))
    {
        atomicAdd(pushed, 1);
    }
}

static int
sum_of(const int* d, int n)
{
    auto h = to_host(d, n);
    int s = 0;
    for (int x : h)
    {
        s += x;
    }
    return s;
}

// An allocator type of the caller's, as the reference's custom_allocator tests use
// (tests/stdgpu/unordered_datastructure.inc:2510-2548): the containers accept and return it.
template <typename T>
struct tagged_allocator : stdgpu::safe_device_allocator<T>
{
    using value_type = T;
    int tag = 0;
    tagged_allocator() = default;
    explicit tagged_allocator(int t)
      : tag(t)
    {
    }
    template <typename U>
    tagged_allocator(const tagged_allocator<U>& o)
      : tag(o.tag)
    {
    }
};

// vector / deque device element access and the other device calls of the reference's containers
__global__ void
vector_pop(stdgpu::vector<std::uint32_t> v, int n, std::uint32_t* popped, int* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        const auto r = v.pop_back();
        popped[i] = r.first;
        ok[i] = r.second ? 1 : 0;
    }
}

__global__ void
vector_peek(stdgpu::vector<std::uint32_t> v, std::uint32_t* out)
{
    out[0] = v.front();
    out[1] = v.back();
    out[2] = v.at(3);
    out[3] = v[4];
    out[4] = v.emplace_back(777u) ? 1u : 0u;
}

__global__ void
deque_sequence(stdgpu::deque<std::uint64_t> d, int n, std::uint64_t* out)
{
    // one thread: pushes in program order, then reads the ends and one element by index
    for (int i = 0; i < n; ++i)
    {
        d.emplace_back(static_cast<std::uint64_t>(1000 + i));
    }
    out[0] = d.front();
    out[1] = d.back();
    out[2] = d.at(7);
    out[3] = d[n - 2];
}

int
main()
{
    std::setvbuf(stdout, nullptr, _IOLBF, 0); // each line out before a failure can end the program
    const int N = 100000;
    const int threads = 256;
    const int blocks = (N + threads - 1) / threads;
    auto keys = unique_keys(N, 42);
    std::uint64_t* d_keys = to_device(keys);
    int* flags = nullptr;
    int* flags2 = nullptr;
    cudaMalloc(&flags, sizeof(int) * N);
    cudaMalloc(&flags2, sizeof(int) * N);
    unsigned long long* d_sum = nullptr;
    cudaMalloc(&d_sum, sizeof(unsigned long long));

    // insert_unique_parallel (unordered_datastructure.inc:1880)
    {
        map_t m = map_t::createDeviceObject(N);
        k_insert<<<blocks, threads>>>(m, d_keys, N, flags);
        check(sum_of(flags, N) == N, "insert_unique_parallel: every key inserted once");
        check(m.size() == N && m.valid(), "insert_unique_parallel: size and valid");
        k_find_values<<<blocks, threads>>>(m, d_keys, N, flags);
        check(sum_of(flags, N) == N, "find returns the stored pair");
        cudaMemset(d_sum, 0, sizeof(unsigned long long));
        k_count_sum<<<blocks, threads>>>(m, d_keys, N, d_sum);
        check(to_host(d_sum, 1)[0] == static_cast<unsigned long long>(N), "count_sum");
        cudaMemset(d_sum, 0, sizeof(unsigned long long));
        k_bucket_size_sum<<<(m.bucket_count() + threads - 1) / threads, threads>>>(m, d_sum);
        check(to_host(d_sum, 1)[0] == static_cast<unsigned long long>(N), "bucket_size_sum");
        auto r = m.device_range();
        cudaMemset(d_sum, 0, sizeof(unsigned long long));
        k_range_sum<<<(r.size() + threads - 1) / threads, threads>>>(r, d_sum);
        check(r.size() == N && to_host(d_sum, 1)[0] == static_cast<unsigned long long>(N) * (N - 1) / 2,
              "device_range covers every stored pair");
        // erase_unique_parallel (unordered_datastructure.inc:1898)
        k_erase<<<blocks, threads>>>(m, d_keys, N, flags);
        check(sum_of(flags, N) == N && m.size() == 0 && m.empty() && m.valid(), "erase_unique_parallel");
        // a second erase finds nothing
        k_erase<<<blocks, threads>>>(m, d_keys, N, flags);
        check(sum_of(flags, N) == 0, "erase of absent keys");
        map_t::destroyDeviceObject(m);
    }

    // emplace_unique_parallel, then the bulk calls on the same object
    {
        map_t m = map_t::createDeviceObject(N);
        k_emplace<<<blocks, threads>>>(m, d_keys, N, flags);
        check(sum_of(flags, N) == N && m.size() == N, "emplace_unique_parallel");
        k_emplace<<<blocks, threads>>>(m, d_keys, N, flags);
        check(sum_of(flags, N) == 0 && m.size() == N, "emplace of present keys inserts nothing");
        m.clear();
        check(m.size() == 0 && m.valid(), "clear");
        // bulk insert(begin, end) over value_type elements (unordered_base_detail.cuh:996-1017)
        std::vector<map_t::value_type> values;
        values.reserve(N);
        for (int i = 0; i < N; ++i)
        {
            values.emplace_back(keys[i], static_cast<std::uint32_t>(i));
        }
        map_t::value_type* d_values = nullptr;
        cudaMalloc(&d_values, sizeof(map_t::value_type) * N);
        cudaMemcpy(d_values, values.data(), sizeof(map_t::value_type) * N, cudaMemcpyHostToDevice);
        m.insert(d_values, d_values + N);
        k_find_values<<<blocks, threads>>>(m, d_keys, N, flags);
        check(m.size() == N && sum_of(flags, N) == N, "bulk insert(begin, end)");
        m.erase(d_keys, d_keys + N / 2);
        check(m.size() == N - N / 2 && m.valid(), "bulk erase(begin, end)");
        cudaFree(d_values);
        map_t::destroyDeviceObject(m);
    }

    // device find in every call shape against the host model: full warps, odd lanes only, out-of-band and
    // absent keys mixed into full warps
    {
        const int n = 4096;
        map_t m = map_t::createDeviceObject(n);
        std::vector<std::uint64_t> k(n);
        std::vector<std::uint32_t> want(n, 0u);
        std::vector<stdgpu::pair<const std::uint64_t, std::uint32_t>> stored;
        for (int i = 0; i < n; ++i)
        {
            k[i] = i % 97 == 5 ? ~0ull : (i % 89 == 7 ? ~0ull - 1 : keys[i]);
            if (i % 3 != 0) // two keys in three are stored, with value i
            {
                want[i] = static_cast<std::uint32_t>(i) + 1u;
            }
        }
        // the out-of-band keys are stored once each, with the value of their first stored occurrence
        std::unordered_map<std::uint64_t, std::uint32_t> first;
        for (int i = 0; i < n; ++i)
        {
            if (want[i] != 0u && first.emplace(k[i], static_cast<std::uint32_t>(i)).second)
            {
                stored.emplace_back(k[i], static_cast<std::uint32_t>(i));
            }
        }
        for (int i = 0; i < n; ++i)
        {
            auto f = first.find(k[i]);
            want[i] = f != first.end() ? f->second + 1u : 0u;
        }
        auto* dv = to_device(stored);
        m.insert(dv, dv + stored.size());
        auto* dk = to_device(k);
        auto* dw = to_device(want);
        int* dbad = nullptr;
        cudaMalloc(&dbad, sizeof(int));
        bool ok = true;
        for (int mode = 0; mode < 2; ++mode)
        {
            cudaMemset(dbad, 0, sizeof(int));
            k_find_shapes<<<(n + 127) / 128, 128>>>(m, dk, dw, n, mode, dbad);
            ok = ok && to_host(dbad, 1)[0] == 0;
        }
        check(ok && m.size() == static_cast<stdgpu::index_t>(stored.size()),
              "device find: full warps, half warps, out-of-band and absent keys");
        cudaFree(dv);
        cudaFree(dk);
        cudaFree(dw);
        cudaFree(dbad);
        map_t::destroyDeviceObject(m);
    }

    // insert_and_erase_unique_parallel (unordered_datastructure.inc:2118)
    {
        const int n = 10000;
        map_t m = map_t::createDeviceObject(N);
        k_insert_and_erase<<<(n + threads - 1) / threads, threads>>>(m, d_keys, n, flags, flags2);
        check(sum_of(flags, n) == n && sum_of(flags2, n) == n && m.size() == 0 && m.valid(),
              "insert_and_erase_unique_parallel");
        map_t::destroyDeviceObject(m);
    }

    // insert_parallel_while_one_free (unordered_datastructure.inc:1549): capacity 1 gives 2 slots
    {
        set_t s = set_t::createDeviceObject(1);
        check(s.max_size() == 2 && s.bucket_count() == 1, "capacity 1 geometry");
        k_insert_same<<<1, 1>>>(s, 11, 1, flags);
        k_insert_same<<<blocks, threads>>>(s, 22, N, flags);
        check(sum_of(flags, N) == 1 && s.size() == 2 && s.full() && s.valid(), "insert_parallel_while_one_free");
        k_insert_same<<<blocks, threads>>>(s, 33, N, flags);
        check(sum_of(flags, N) == 0 && s.size() == 2, "insert_multiple_while_full");
        set_t::destroyDeviceObject(s);
    }

    // insert_while_excess_empty below max_size(): capacity 3 has 7 slots, but the reference refuses once its
    // excess list (3 slots) is empty.  Keys and outcomes recorded from the reference (tests/golden/refusal.npz,
    // capacity 3), one device insert per launch in that order; then 10^5 device inserts of a new key are all
    // refused.
    {
        const std::uint64_t keys3[16] = { 1638364144ull,   1070330891283ull, 328095614449ull,  345231260195ull,
                                          980446690571ull, 643393456553ull,  518210457150ull,  850227063600ull,
                                          33365788281ull,  777316343105ull,  411485446533ull,  99893614912ull,
                                          726227504283ull, 1024155339141ull, 227809098477ull,  692791501211ull };
        const int expect3[16] = { 1, 1, 1, 1, 1, 1, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0 };
        set_t s = set_t::createDeviceObject(3);
        check(s.max_size() == 7, "capacity 3 geometry");
        bool same = true;
        for (int i = 0; i < 16; ++i)
        {
            k_insert_same<<<1, 1>>>(s, keys3[i], 1, flags);
            same = same && to_host(flags, 1)[0] == expect3[i];
        }
        check(same && s.size() == 6 && !s.full() && s.valid(), "insert_while_excess_empty (device inserts, capacity 3)");
        k_insert_same<<<blocks, threads>>>(s, 1ull << 40, N, flags);
        check(sum_of(flags, N) == 0 && s.size() == 6 && s.valid(), "insert_parallel_while_excess_empty");
        set_t::destroyDeviceObject(s);
    }

    // vector push_back from a user kernel (tests/stdgpu/vector.inc:404-512)
    {
        stdgpu::vector<std::uint32_t> v = stdgpu::vector<std::uint32_t>::createDeviceObject(N);
        cudaMemset(flags, 0, sizeof(int) * N);
        k_push_if<<<blocks, threads>>>(v, N, flags);
        const int expected = (N + 2) / 3;
        auto data = to_host(v.data(), expected);
        long long sum = 0;
        for (auto x : data)
        {
            sum += x;
        }
        long long want = 0;
        for (int i = 0; i < N; i += 3)
        {
            want += i;
        }
        check(v.size() == expected && sum_of(flags, N) == expected && sum == want, "vector push_back in a kernel");
        stdgpu::vector<std::uint32_t>::destroyDeviceObject(v);
    }

    // bitset count
    {
        std::vector<std::uint32_t> words(1000);
        std::mt19937 rng(3);
        long long want = 0;
        for (auto& w : words)
        {
            w = rng();
            want += __builtin_popcount(w);
        }
        std::uint32_t* d_words = to_device(words);
        check(stdgpu::bitset_count(d_words, 32000) == want, "bitset count");
        cudaFree(d_words);
    }

    // deque: device push_back / pop_front from one launch, then FIFO order across launches
    {
        const int n = 1 << 16;
        auto d = stdgpu::deque<std::uint64_t>::createDeviceObject(n);
        std::vector<std::uint64_t> v(n);
        for (int i = 0; i < n; ++i)
        {
            v[i] = 1000000ull + static_cast<std::uint64_t>(i);
        }
        std::uint64_t* d_v = to_device(v);
        std::uint64_t* d_p = nullptr;
        std::uint8_t* d_ok = nullptr;
        cudaMalloc(&d_p, sizeof(std::uint64_t) * n);
        cudaMalloc(&d_ok, n);
        deque_fill<<<(n / 2 + 255) / 256, 256>>>(d, d_v, n / 2, d_ok); // first half of the values, in one launch
        check(d.size() == n / 2 && count_ok(d_ok, n / 2) == n / 2, "deque push_back from a kernel");
        deque_mixed<<<(n + 255) / 256, 256>>>(d, d_v + n / 2 - 1, n, d_p, d_ok);
        auto ok = to_host(d_ok, n);
        auto popped = to_host(d_p, n);
        std::multiset<std::uint64_t> out, in;
        long long pushes = 0, pops = 0;
        for (int i = 0; i < n; ++i)
        {
            if (i & 1)
            {
                pops += ok[i];
                if (ok[i])
                {
                    out.insert(popped[i]);
                }
            }
            else
            {
                pushes += ok[i];
            }
        }
        // everything popped was in the deque before the launch or pushed during it
        for (int i = 0; i < n / 2; ++i)
        {
            in.insert(v[i]);
        }
        for (int i = 0; i < n; i += 2)
        {
            if (ok[i])
            {
                in.insert(v[n / 2 - 1 + i]);
            }
        }
        bool sub = true;
        for (auto x : out)
        {
            auto it = in.find(x);
            sub = sub && it != in.end();
            if (it != in.end())
            {
                in.erase(it);
            }
        }
        check(sub && d.size() == n / 2 + pushes - pops, "deque mixed push_back / pop_front: conservation");
        // drain: what is left comes out, and a second drain finds it empty
        const stdgpu::index_t left = d.size();
        deque_drain<<<(n + 255) / 256, 256>>>(d, n, d_p, d_ok);
        check(count_ok(d_ok, n) == left && d.empty(), "deque drain");
        stdgpu::deque<std::uint64_t>::destroyDeviceObject(d);
        cudaFree(d_v);
        cudaFree(d_p);
        cudaFree(d_ok);

        auto q = stdgpu::queue<std::uint32_t>::createDeviceObject(1000);
        int* d_pushed = nullptr;
        cudaMalloc(&d_pushed, sizeof(int));
        cudaMemset(d_pushed, 0, sizeof(int));
        queue_push<<<8, 256>>>(q, 2048, d_pushed);
        check(to_host(d_pushed, 1)[0] == 1000 && q.size() == 1000, "queue push stops at capacity");
        stdgpu::queue<std::uint32_t>::destroyDeviceObject(q);
        cudaFree(d_pushed);
    }

    // empty_container (unordered_datastructure.inc:72-80): a default-constructed object
    {
        map_t empty_container;
        check(empty_container.empty() && empty_container.full() && empty_container.size() == 0 &&
                      empty_container.valid(),
              "empty_container");
        stdgpu::vector<std::uint32_t> v;
        stdgpu::deque<std::uint64_t> d;
        check(v.size() == 0 && d.size() == 0, "default-constructed vector / deque hold nothing");
    }

    // empty_size_limits and the custom-execution-policy variant (unordered_datastructure.inc:249-265),
    // hash_objects (:267-279), hash_inside_range (:84-108)
    {
        cudaStream_t st = nullptr;
        cudaStreamCreate(&st);
        const auto policy = stdgpu::execution::on(st);
        map_t m = map_t::createDeviceObject(policy, N);
        check(m.empty() && !m.full() && m.size() <= m.max_size() && m.load_factor() <= m.max_load_factor(),
              "empty_size_limits");
        check(m.empty(policy) && !m.full(policy) && m.size(policy) <= m.max_size() &&
                      m.load_factor(policy) <= m.max_load_factor(),
              "empty_size_limits_custom_execution_policy");
        const std::uint64_t key = 0x1234567890ull;
        check(m.key_eq()(key, key) && m.hash_function()(key) == m.hash_function()(key), "hash_objects");
        bool inside = true;
        std::uint64_t x = 88172645463325252ull;
        for (int i = 0; i < (1 << 16); ++i)
        {
            x ^= x << 13;
            x ^= x >> 7;
            x ^= x << 17;
            const stdgpu::index_t b = m.bucket(x);
            inside = inside && b >= 0 && b < m.bucket_count();
        }
        check(inside, "hash_inside_range");
        // insert_range / erase_range / clear with a custom execution policy (unordered_datastructure.inc:1933,
        // :2015, :2494)
        std::vector<map_t::value_type> values;
        values.reserve(N);
        for (int i = 0; i < N; ++i)
        {
            values.emplace_back(keys[i], static_cast<std::uint32_t>(i));
        }
        map_t::value_type* d_values = nullptr;
        cudaMalloc(&d_values, sizeof(map_t::value_type) * N);
        cudaMemcpy(d_values, values.data(), sizeof(map_t::value_type) * N, cudaMemcpyHostToDevice);
        m.insert(policy, d_values, d_values + N);
        check(m.size(policy) == N && m.valid(policy), "insert_range_unique_parallel_custom_execution_policy");
        m.erase(policy, d_keys, d_keys + N);
        check(m.size(policy) == 0 && m.valid(policy), "erase_range_unique_parallel_custom_execution_policy");
        m.insert(policy, d_values, d_values + N);
        m.clear(policy);
        check(m.size(policy) == 0 && m.valid(policy), "clear_custom_execution_policy");
        map_t::destroyDeviceObject(policy, m);
        cudaFree(d_values);
        cudaStreamDestroy(st);
    }

    // vector: range insert / erase at the end, device pop_back / element access / emplace_back, valid, clear
    // (vector.inc scenarios on insert, erase, pop_back, front / back / at)
    {
        using vec_t = stdgpu::vector<std::uint32_t>;
        vec_t v = vec_t::createDeviceObject(100);
        std::vector<std::uint32_t> h(60);
        for (int i = 0; i < 60; ++i)
        {
            h[i] = static_cast<std::uint32_t>(10 * i);
        }
        std::uint32_t* d_h = to_device(h);
        v.insert(v.device_end(), d_h, d_h + 50);
        check(v.size() == 50 && v.valid(), "vector insert(device_end(), begin, end)");
        v.insert(v.device_end(), d_h, d_h + 60);
        check(v.size() == 50, "vector insert that would overflow inserts nothing");
        auto r = v.device_range();
        check(r.size() == 50 && to_host(r.begin(), 50) == std::vector<std::uint32_t>(h.begin(), h.begin() + 50),
              "vector device_range()");
        v.erase(v.device_end() - 20, v.device_end());
        check(v.size() == 30 && v.valid(), "vector erase(device_end() - 20, device_end())");
        std::uint32_t* d_out = nullptr;
        int* d_ok = nullptr;
        cudaMalloc(&d_out, sizeof(std::uint32_t) * 64);
        cudaMalloc(&d_ok, sizeof(int) * 64);
        vector_peek<<<1, 1>>>(v, d_out);
        const auto peek = to_host(d_out, 5);
        check(peek[0] == 0 && peek[1] == 290 && peek[2] == 30 && peek[3] == 40 && peek[4] == 1 && v.size() == 31,
              "vector front / back / at / operator[] / emplace_back");
        vector_pop<<<1, 64>>>(v, 40, d_out, d_ok);
        const auto popped = to_host(d_out, 40);
        const auto okv = to_host(d_ok, 40);
        std::vector<std::uint32_t> got;
        for (int i = 0; i < 40; ++i)
        {
            if (okv[i])
            {
                got.push_back(popped[i]);
            }
        }
        std::sort(got.begin(), got.end());
        std::vector<std::uint32_t> want(h.begin(), h.begin() + 30);
        want.push_back(777u);
        std::sort(want.begin(), want.end());
        check(got == want && v.size() == 0 && v.empty() && v.valid(),
              "vector pop_back: each element once, then fails on empty");
        v.insert(v.device_end(), d_h, d_h + 10);
        v.clear();
        check(v.size() == 0 && v.valid(), "vector clear");
        vec_t::destroyDeviceObject(v);
        cudaFree(d_h);
        cudaFree(d_out);
        cudaFree(d_ok);
    }

    // vector: push_back and pop_back in one launch (vector.inc:1022-1056, N = 100000), then the same on a
    // vector that a bulk call left non-empty, and a second launch on the result
    {
        using ivec = stdgpu::vector<int>;
        const int N = 100000;
        ivec pool = ivec::createDeviceObject(N);
        ivec validation = ivec::createDeviceObject(N);
        std::vector<int> h(N);
        for (int i = 0; i < N; ++i)
        {
            h[i] = i + 1;
        }
        int* d_v = to_device(h);
        vector_push_then_pop<<<(N + 127) / 128, 128>>>(pool, validation, d_v, N);
        std::vector<int> got = to_host(validation.data(), N);
        std::sort(got.begin(), got.end());
        check(pool.size() == 0 && pool.empty() && !pool.full() && pool.valid() && validation.size() == N &&
                      validation.full() && validation.valid() && got == h,
              "vector simultaneous_push_back_and_pop_back");
        // the pool starts from 5000 elements inserted by a bulk call: the launch's pops may take those too
        pool.insert(pool.device_end(), d_v, d_v + 5000);
        validation.clear();
        vector_push_then_pop<<<(N / 2 + 127) / 128, 128>>>(pool, validation, d_v + 5000, N / 2);
        const int left = pool.size();
        std::vector<int> all = to_host(validation.data(), validation.size());
        std::vector<int> rest = to_host(pool.data(), left);
        all.insert(all.end(), rest.begin(), rest.end());
        std::sort(all.begin(), all.end());
        std::vector<int> want(h.begin(), h.begin() + 5000 + N / 2);
        check(left == 5000 && validation.size() == N / 2 && all == want && pool.valid() && validation.valid(),
              "vector push_back and pop_back in one launch after a bulk insert: every element kept once");
        ivec::destroyDeviceObject(pool);
        ivec::destroyDeviceObject(validation);
        cudaFree(d_v);
    }

    // deque: the reference's simultaneous_* scenarios (deque.inc:1494-1700, N = 100000) for all four pairs
    // of ends, the *_some / *_all / *_too_many scenarios of push_front, emplace_front and pop_back
    // (deque.inc:284-345, 962-1245), push_front_circular (deque.inc:1298-1336), and a bulk call after
    // device calls (turn words rebuilt)
    {
        using idq = stdgpu::deque<int>;
        const int N = 100000;
        std::vector<int> h(N);
        for (int i = 0; i < N; ++i)
        {
            h[i] = i + 1;
        }
        int* d_v = to_device(h);
        const char* names[4] = { "deque simultaneous_push_back_and_pop_back", "deque simultaneous_push_front_and_pop_back",
                                 "deque simultaneous_push_back_and_pop_front",
                                 "deque simultaneous_push_front_and_pop_front" };
        for (int mode = 0; mode < 4; ++mode)
        {
            idq pool = idq::createDeviceObject(N);
            idq validation = idq::createDeviceObject(N);
            deque_push_then_pop<<<(N + 127) / 128, 128>>>(pool, validation, d_v, N, mode);
            auto r = validation.device_range();
            std::vector<int> got = to_host(r.begin(), r.size());
            std::sort(got.begin(), got.end());
            check(pool.size() == 0 && pool.empty() && !pool.full() && pool.valid() && validation.size() == N &&
                          validation.full() && validation.valid() && got == h,
                  names[mode]);
            idq::destroyDeviceObject(pool);
            idq::destroyDeviceObject(validation);
        }
        int* d_ok = nullptr;
        cudaMalloc(&d_ok, sizeof(int) * N);
        // the reference's fill_deque (deque.inc:206-227): device push_back of 1..n, then the storage sorted so
        // that element i holds i + 1
        auto fill_sorted = [&](idq& d, int n) {
            deque_calls<<<(n + 127) / 128, 128>>>(d, d_v, n, 0, d_ok);
            std::vector<int> st = to_host(d.data(), n);
            std::sort(st.begin(), st.end());
            cudaMemcpy(d.data(), st.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
        };
        auto ok_count = [&](int n) {
            long long c = 0;
            for (int x : to_host(d_ok, n))
            {
                c += x;
            }
            return c;
        };
        // push_front / emplace_front: some, all, too many
        for (int op = 1; op <= 2; ++op)
        {
            const int M = 10000;
            const int sizes[3] = { M / 2, M, M + 500 };
            for (int k = 0; k < 3; ++k)
            {
                idq d = idq::createDeviceObject(M);
                deque_calls<<<(sizes[k] + 127) / 128, 128>>>(d, d_v, sizes[k], op, d_ok);
                const int want = sizes[k] < M ? sizes[k] : M;
                auto r = d.device_range();
                std::vector<int> got = to_host(r.begin(), r.size());
                std::sort(got.begin(), got.end());
                bool vals = static_cast<int>(got.size()) == want;
                for (int i = 0; vals && i + 1 < want; ++i)
                {
                    vals = got[i] < got[i + 1] && got[i] >= 1 && got[i + 1] <= sizes[k];
                }
                check(ok_count(sizes[k]) == want && d.size() == want && d.valid() && vals,
                      std::string(op == 1 ? "deque push_front" : "deque emplace_front") +
                              (k == 0 ? "_some" : k == 1 ? "_all" : "_too_many"));
                idq::destroyDeviceObject(d);
            }
        }
        // pop_back: some, all, too many, from a deque filled by push_back 1..M; the back elements go first
        {
            const int M = 10000;
            const int pops[3] = { M / 3, M, M + 700 };
            for (int k = 0; k < 3; ++k)
            {
                idq d = idq::createDeviceObject(M);
                fill_sorted(d, M);
                deque_calls<<<(pops[k] + 127) / 128, 128>>>(d, d_v, pops[k], 3, d_ok);
                const int taken = pops[k] < M ? pops[k] : M;
                auto r = d.device_range();
                std::vector<int> left = to_host(r.begin(), r.size());
                std::sort(left.begin(), left.end());
                std::vector<int> want(h.begin(), h.begin() + (M - taken));
                check(ok_count(pops[k]) == taken && d.size() == M - taken && d.valid() && left == want,
                      std::string("deque pop_back") + (k == 0 ? "_some" : k == 1 ? "_all" : "_too_many"));
                idq::destroyDeviceObject(d);
            }
        }
        // push_front_circular: fill 1..M, pop_back M/3, pop_front M/3, push_front 2M/3 new values
        {
            const int M = 10000;
            const int n_pop = M / 3;
            const int n_push = 2 * n_pop;
            idq d = idq::createDeviceObject(M);
            fill_sorted(d, M);
            deque_calls<<<(n_pop + 127) / 128, 128>>>(d, d_v, n_pop, 3, d_ok);
            deque_calls<<<(n_pop + 127) / 128, 128>>>(d, d_v, n_pop, 4, d_ok);
            deque_calls<<<(n_push + 127) / 128, 128>>>(d, d_v + M - n_pop, n_push, 1, d_ok);
            auto r = d.device_range();
            std::vector<int> got = to_host(r.begin(), r.size());
            std::sort(got.begin(), got.end());
            std::vector<int> want;
            for (int i = 0; i < M - 2 * n_pop; ++i)
            {
                want.push_back(n_pop + 1 + i);
            }
            for (int i = 0; i < n_push; ++i)
            {
                want.push_back(M - n_pop + 1 + i);
            }
            std::sort(want.begin(), want.end());
            check(d.size() == M - 2 * n_pop + n_push && d.valid() && got == want, "deque push_front_circular");
            // a bulk call after the device calls: pop_front of everything through the host, front to back
            std::uint8_t* d_bok = nullptr;
            int* d_pop = nullptr;
            const int n_all = M - 2 * n_pop + n_push;
            cudaMalloc(&d_bok, n_all);
            cudaMalloc(&d_pop, sizeof(int) * n_all);
            std::vector<std::uint8_t> is_push(n_all, 0);
            std::uint8_t* d_is_push = to_device(is_push);
            check(sg_deque_ops(d.native_handle(), d_is_push, nullptr, n_all, d_pop, d_bok, nullptr) == SG_OK,
                  "deque bulk call after device calls: accepted");
            std::vector<int> popped_all = to_host(d_pop, n_all);
            std::sort(popped_all.begin(), popped_all.end());
            check(count_ok(d_bok, n_all) == n_all && d.size() == 0 && d.valid() && popped_all == want,
                  "deque bulk pop_front after device calls: every element once");
            cudaFree(d_bok);
            cudaFree(d_pop);
            cudaFree(d_is_push);
            idq::destroyDeviceObject(d);
        }
        cudaFree(d_ok);
        cudaFree(d_v);
    }

    // deque: device emplace_back, front / back / at / operator[], device_range, valid, max_size
    {
        using dq_t = stdgpu::deque<std::uint64_t>;
        dq_t d = dq_t::createDeviceObject(64);
        std::uint64_t* d_out = nullptr;
        cudaMalloc(&d_out, sizeof(std::uint64_t) * 4);
        deque_sequence<<<1, 1>>>(d, 40, d_out);
        const auto out = to_host(d_out, 4);
        check(out[0] == 1000 && out[1] == 1039 && out[2] == 1007 && out[3] == 1038 && d.size() == 40 && d.valid() &&
                      d.max_size() == 64,
              "deque emplace_back / front / back / at / operator[]");
        auto r = d.device_range();
        const auto all = to_host(r.begin(), r.size());
        bool in_order = r.size() == 40;
        for (int i = 0; in_order && i < 40; ++i)
        {
            in_order = all[i] == static_cast<std::uint64_t>(1000 + i);
        }
        check(in_order, "deque device_range(): front to back");
        dq_t::destroyDeviceObject(d);
        cudaFree(d_out);
    }

    // get_allocator and custom_allocator (unordered_datastructure.inc:2510-2548)
    {
        using alloc_t = tagged_allocator<map_t::value_type>;
        using custom_map_t = stdgpu::unordered_map<std::uint64_t, std::uint32_t, stdgpu::hash<std::uint64_t>,
                                                   stdgpu::equal_to<std::uint64_t>, alloc_t>;
        custom_map_t m = custom_map_t::createDeviceObject(10000, alloc_t(7));
        alloc_t a = m.get_allocator();
        custom_map_t::value_type* array = a.allocate(10000);
        const bool allocated = array != nullptr && cudaMemset(array, 0, sizeof(*array) * 10000) == cudaSuccess;
        a.deallocate(array, 10000);
        map_t plain = map_t::createDeviceObject(100);
        auto pa = plain.get_allocator();
        map_t::value_type* parray = pa.allocate(100);
        pa.deallocate(parray, 100);
        check(a.tag == 7 && allocated && parray != nullptr && m.size() == 0 && m.valid(),
              "get_allocator / custom_allocator");
        custom_map_t::destroyDeviceObject(m);
        map_t::destroyDeviceObject(plain);
        stdgpu::vector<std::uint32_t, tagged_allocator<std::uint32_t>> v =
                stdgpu::vector<std::uint32_t, tagged_allocator<std::uint32_t>>::createDeviceObject(16);
        check(v.capacity() == 16 && v.get_allocator().tag == 0, "vector with an allocator type");
        stdgpu::vector<std::uint32_t, tagged_allocator<std::uint32_t>>::destroyDeviceObject(v);
    }

    cudaError_t e = cudaDeviceSynchronize();
    check(e == cudaSuccess, "no CUDA error");
    cudaFree(d_keys);
    cudaFree(flags);
    cudaFree(flags2);
    cudaFree(d_sum);
    if (failures == 0)
    {
        std::printf("ALL PASS\n");
        return 0;
    }
    std::printf("%d FAILED\n", failures);
    return 1;
}

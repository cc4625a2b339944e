// Device-side insert / erase churn on tiny tables: the pattern of a caller that allocates and frees entries
// from its own kernels for many launches (the reference's device insert reuses the slots erase frees,
// src/stdgpu/impl/unordered_base_detail.cuh:708-809, 811-913, 958-994).  Every launch inserts and erases
// keys of a small key set with several threads per key; inserts and erases of different keys share a
// launch.  After every launch the per-key outcomes and size() match a std::unordered_set /
// std::unordered_map model, and no insert of an absent key is refused while the table holds fewer than
// max_size() keys (part 1 keeps fewer live keys than the reference's excess list has slots; parts 1b and 3
// switch the excess-list accounting off, so their tables take keys up to max_size()).  A second part races
// inserts and erases of the same keys in one launch and checks the invariants that hold for any
// interleaving; a third fills the table to max_size() through churn.
//
// usage: device_churn_test [out_dir]  -- with out_dir, the launches of the first part (keys and per-thread
// outcomes) are written there for a replay on the oracle.  Prints one line per check and "ALL PASS".
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <random>
#include <string>
#include <unordered_map>
#include <unordered_set>
#include <vector>

#include <stdgpu_gb300/stdgpu.cuh>

using set_t = stdgpu::unordered_set<std::uint64_t>;
using map_t = stdgpu::unordered_map<std::uint64_t, std::uint32_t>;

static int failures = 0;

static void
check(bool ok, const std::string& name)
{
    if (!ok)
    {
        std::printf("FAIL %s\n", name.c_str());
        ++failures;
    }
}

template <typename T>
static T*
to_device(const std::vector<T>& h)
{
    T* d = nullptr;
    cudaMalloc(&d, sizeof(T) * (h.empty() ? 1 : h.size()));
    if (!h.empty())
    {
        cudaMemcpy(d, h.data(), sizeof(T) * h.size(), cudaMemcpyHostToDevice);
    }
    return d;
}

template <typename T>
static std::vector<T>
to_host(const T* d, size_t n)
{
    std::vector<T> h(n);
    if (n != 0)
    {
        cudaMemcpy(h.data(), d, sizeof(T) * n, cudaMemcpyDeviceToHost);
    }
    return h;
}

// threads [0, n_ins) insert keys[i], threads [n_ins, n) erase keys[i]
__global__ void
k_churn_set(set_t s, const std::uint64_t* keys, int n_ins, int n, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        ok[i] = i < n_ins ? (s.insert(keys[i]).second ? 1 : 0) : (s.erase(keys[i]) == 1 ? 1 : 0);
    }
}

__global__ void
k_churn_map(map_t m, const std::uint64_t* keys, const std::uint32_t* vals, int n_ins, int n, std::uint8_t* ok)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        ok[i] = i < n_ins ? (m.emplace(keys[i], vals[i]).second ? 1 : 0) : (m.erase(keys[i]) == 1 ? 1 : 0);
    }
}

__global__ void
k_find_map(map_t m, const std::uint64_t* keys, int n, std::uint8_t* found, std::uint32_t* vals)
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
k_contains(set_t s, const std::uint64_t* keys, int n, std::uint8_t* found)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n)
    {
        found[i] = s.contains(keys[i]) ? 1 : 0;
    }
}

struct launch
{
    std::vector<std::uint64_t> keys;
    int n_ins = 0;
};

// A launch over the key set: some absent keys inserted and some present keys erased, each by 1-4 threads,
// no key both inserted and erased; plus inserts of present keys and erases of absent ones (no-ops).
static launch
make_launch(std::mt19937_64& rng, const std::vector<std::uint64_t>& universe, const std::unordered_set<std::uint64_t>& model,
            double p_ins, double p_er)
{
    launch L;
    std::vector<std::uint64_t> ins, er;
    std::uniform_real_distribution<double> u(0.0, 1.0);
    for (std::uint64_t k : universe)
    {
        const bool present = model.count(k) != 0;
        const double x = u(rng);
        const int copies = 1 + static_cast<int>(rng() % 4);
        if ((!present && x < p_ins) || (present && x < 0.1))
        {
            for (int c = 0; c < copies; ++c)
            {
                ins.push_back(k);
            }
        }
        else if ((present && x < 0.1 + p_er) || (!present && x > 0.95))
        {
            for (int c = 0; c < copies; ++c)
            {
                er.push_back(k);
            }
        }
    }
    std::shuffle(ins.begin(), ins.end(), rng);
    std::shuffle(er.begin(), er.end(), rng);
    L.n_ins = static_cast<int>(ins.size());
    L.keys = ins;
    L.keys.insert(L.keys.end(), er.begin(), er.end());
    return L;
}

static void
write_raw(const std::string& path, const void* p, size_t bytes)
{
    FILE* f = std::fopen(path.c_str(), "wb");
    if (f != nullptr)
    {
        std::fwrite(p, 1, bytes, f);
        std::fclose(f);
    }
}

int
main(int argc, char** argv)
{
    const std::string out_dir = argc > 1 ? argv[1] : "";
    std::mt19937_64 rng(2024);

    // ---- part 1: deterministic churn on unordered_set<uint64_t>, capacity 64
    {
        set_t s = set_t::createDeviceObject(64);
        const int max_size = s.max_size();
        // 40 keys: every insert of an absent key needs a free slot, so a table that never reused erased
        // slots would refuse after its max_size() never-used slots are gone (a few launches); and with at
        // most 40 keys live the reference's own excess list (42 entries at this capacity) is never exhausted,
        // so its replay refuses nothing either
        std::vector<std::uint64_t> universe;
        for (int i = 0; i < 40; ++i)
        {
            universe.push_back((rng() >> 4) | 1u);
        }
        std::unordered_set<std::uint64_t> model;
        std::vector<std::int32_t> meta; // per launch: n, n_ins
        std::vector<std::uint64_t> all_keys;
        std::vector<std::uint8_t> all_ok;
        bool sizes_ok = true, outcomes_ok = true, refused = false;
        const int launches = 400;
        for (int l = 0; l < launches; ++l)
        {
            const double p_ins = (l / 40) % 2 == 0 ? 0.6 : 0.2;
            launch L = make_launch(rng, universe, model, p_ins, 0.8 - p_ins);
            const int n = static_cast<int>(L.keys.size());
            std::uint64_t* dk = to_device(L.keys);
            std::uint8_t* dok = nullptr;
            cudaMalloc(&dok, n + 1);
            if (n > 0)
            {
                k_churn_set<<<(n + 127) / 128, 128>>>(s, dk, L.n_ins, n, dok);
            }
            std::vector<std::uint8_t> ok = to_host(dok, n);
            cudaFree(dk);
            cudaFree(dok);
            // per key: successes of its inserts / erases against the model
            std::unordered_map<std::uint64_t, int> ins_ok, er_ok;
            for (int i = 0; i < n; ++i)
            {
                (i < L.n_ins ? ins_ok : er_ok)[L.keys[i]] += ok[i];
            }
            for (const auto& kv : ins_ok)
            {
                const int want = model.count(kv.first) ? 0 : 1;
                outcomes_ok = outcomes_ok && kv.second == want;
                refused = refused || (want == 1 && kv.second == 0);
            }
            for (const auto& kv : er_ok)
            {
                outcomes_ok = outcomes_ok && kv.second == (model.count(kv.first) ? 1 : 0);
            }
            for (const auto& kv : ins_ok)
            {
                model.insert(kv.first);
            }
            for (const auto& kv : er_ok)
            {
                model.erase(kv.first);
            }
            sizes_ok = sizes_ok && s.size() == static_cast<int>(model.size());
            meta.push_back(n);
            meta.push_back(L.n_ins);
            all_keys.insert(all_keys.end(), L.keys.begin(), L.keys.end());
            all_ok.insert(all_ok.end(), ok.begin(), ok.end());
        }
        check(outcomes_ok, "set churn: per-key insert / erase outcomes equal the model in every launch");
        check(!refused, "set churn: no insert of an absent key refused below max_size()");
        check(sizes_ok, "set churn: size() equals the model after every launch");
        check(s.valid(), "set churn: valid()");
        std::vector<std::uint8_t> found(universe.size());
        {
            std::uint64_t* dk = to_device(universe);
            std::uint8_t* df = nullptr;
            cudaMalloc(&df, universe.size());
            k_contains<<<(static_cast<int>(universe.size()) + 127) / 128, 128>>>(s, dk, static_cast<int>(universe.size()), df);
            found = to_host(df, universe.size());
            cudaFree(dk);
            cudaFree(df);
        }
        bool contents = true;
        for (size_t i = 0; i < universe.size(); ++i)
        {
            contents = contents && (found[i] != 0) == (model.count(universe[i]) != 0);
        }
        check(contents, "set churn: final contents equal the model");
        std::printf("set churn: %d launches, %zu operations, max_size %d, final size %zu\n", launches,
                    all_keys.size(), max_size, model.size());
        if (!out_dir.empty())
        {
            const std::int64_t header[2] = { 64, static_cast<std::int64_t>(launches) };
            write_raw(out_dir + "/header.bin", header, sizeof(header));
            write_raw(out_dir + "/meta.bin", meta.data(), meta.size() * sizeof(std::int32_t));
            write_raw(out_dir + "/keys.bin", all_keys.data(), all_keys.size() * sizeof(std::uint64_t));
            write_raw(out_dir + "/ok.bin", all_ok.data(), all_ok.size());
        }
        set_t::destroyDeviceObject(s);
    }

    // ---- part 1b: the same churn on unordered_map<uint64_t, uint32_t>: a re-inserted key takes its new value
    {
        map_t m = map_t::createDeviceObject(100);
        m.set_excess_accounting(false); // keys until no slot is free: up to max_size() - 2 live keys
        const int max_size = m.max_size();
        std::vector<std::uint64_t> universe;
        for (int i = 0; i < max_size - 2; ++i)
        {
            universe.push_back(rng() >> 3);
        }
        std::unordered_map<std::uint64_t, std::uint32_t> model;
        std::unordered_set<std::uint64_t> present;
        bool ok_all = true, refused = false;
        for (int l = 0; l < 300; ++l)
        {
            launch L = make_launch(rng, universe, present, (l / 30) % 2 == 0 ? 0.7 : 0.15, 0.6);
            const int n = static_cast<int>(L.keys.size());
            std::vector<std::uint32_t> vals(n);
            for (int i = 0; i < n; ++i)
            {
                vals[i] = static_cast<std::uint32_t>(L.keys[i] * 2654435761u + static_cast<std::uint64_t>(l));
            }
            std::uint64_t* dk = to_device(L.keys);
            std::uint32_t* dv = to_device(vals);
            std::uint8_t* dok = nullptr;
            cudaMalloc(&dok, n + 1);
            if (n > 0)
            {
                k_churn_map<<<(n + 127) / 128, 128>>>(m, dk, dv, L.n_ins, n, dok);
            }
            std::vector<std::uint8_t> ok = to_host(dok, n);
            cudaFree(dk);
            cudaFree(dv);
            cudaFree(dok);
            std::unordered_map<std::uint64_t, int> ins_ok;
            std::unordered_map<std::uint64_t, std::uint32_t> won;
            for (int i = 0; i < L.n_ins; ++i)
            {
                ins_ok[L.keys[i]] += ok[i];
                if (ok[i])
                {
                    won[L.keys[i]] = vals[i];
                }
            }
            for (const auto& kv : ins_ok)
            {
                const int want = present.count(kv.first) ? 0 : 1;
                ok_all = ok_all && kv.second == want;
                refused = refused || (want == 1 && kv.second == 0);
            }
            for (int i = L.n_ins; i < n; ++i)
            {
                present.erase(L.keys[i]);
                model.erase(L.keys[i]);
            }
            for (const auto& kv : won)
            {
                present.insert(kv.first);
                model[kv.first] = kv.second;
            }
            ok_all = ok_all && m.size() == static_cast<int>(model.size());
        }
        std::uint64_t* dk = to_device(universe);
        std::uint8_t* df = nullptr;
        std::uint32_t* dv = nullptr;
        cudaMalloc(&df, universe.size());
        cudaMalloc(&dv, universe.size() * 4);
        k_find_map<<<(static_cast<int>(universe.size()) + 127) / 128, 128>>>(m, dk, static_cast<int>(universe.size()), df,
                                                                    dv);
        std::vector<std::uint8_t> f = to_host(df, universe.size());
        std::vector<std::uint32_t> v = to_host(dv, universe.size());
        cudaFree(dk);
        cudaFree(df);
        cudaFree(dv);
        bool contents = true;
        for (size_t i = 0; i < universe.size(); ++i)
        {
            auto it = model.find(universe[i]);
            contents = contents && (f[i] != 0) == (it != model.end()) && (it == model.end() || v[i] == it->second);
        }
        check(ok_all, "map churn: per-key outcomes and size() equal the model in every launch");
        check(!refused, "map churn: no insert of an absent key refused below max_size()");
        check(contents && m.valid(), "map churn: find() returns the value of the insert that won; valid()");
        map_t::destroyDeviceObject(m);
    }

    // ---- part 2: inserts and erases of the same keys race in one launch
    {
        set_t s = set_t::createDeviceObject(256);
        std::vector<std::uint64_t> keys;
        for (int i = 0; i < 40; ++i)
        {
            keys.push_back(rng() >> 2);
        }
        bool inv = true;
        std::unordered_set<std::uint64_t> before;
        for (int l = 0; l < 200; ++l)
        {
            // each key: 4 inserts and 3 erases in the same launch, in shuffled thread order
            std::vector<std::uint64_t> ins, er;
            for (std::uint64_t k : keys)
            {
                for (int c = 0; c < 4; ++c)
                {
                    ins.push_back(k);
                }
                for (int c = 0; c < 3; ++c)
                {
                    er.push_back(k);
                }
            }
            std::shuffle(ins.begin(), ins.end(), rng);
            std::shuffle(er.begin(), er.end(), rng);
            std::vector<std::uint64_t> all(ins);
            all.insert(all.end(), er.begin(), er.end());
            const int n = static_cast<int>(all.size());
            std::uint64_t* dk = to_device(all);
            std::uint8_t* dok = nullptr;
            cudaMalloc(&dok, n);
            k_churn_set<<<(n + 63) / 64, 64>>>(s, dk, static_cast<int>(ins.size()), n, dok);
            std::vector<std::uint8_t> ok = to_host(dok, n);
            std::uint8_t* df = nullptr;
            cudaMalloc(&df, keys.size());
            std::uint64_t* dkeys = to_device(keys);
            k_contains<<<(static_cast<int>(keys.size()) + 63) / 64, 64>>>(s, dkeys, static_cast<int>(keys.size()), df);
            std::vector<std::uint8_t> found = to_host(df, keys.size());
            cudaFree(dk);
            cudaFree(dok);
            cudaFree(df);
            cudaFree(dkeys);
            std::unordered_map<std::uint64_t, int> net;
            for (int i = 0; i < n; ++i)
            {
                net[all[i]] += i < static_cast<int>(ins.size()) ? ok[i] : -static_cast<int>(ok[i]);
            }
            std::unordered_set<std::uint64_t> after;
            int n_present = 0;
            for (size_t j = 0; j < keys.size(); ++j)
            {
                // present afterwards exactly when (present before) + successful inserts - successful erases is 1
                const int x = (before.count(keys[j]) ? 1 : 0) + net[keys[j]];
                inv = inv && (x == 0 || x == 1) && (x == 1) == (found[j] != 0);
                if (found[j])
                {
                    after.insert(keys[j]);
                    ++n_present;
                }
            }
            inv = inv && s.size() == n_present;
            before = after;
        }
        check(inv, "racing inserts and erases of one key: one stored copy at most, outcomes consistent with it");
        check(s.valid(), "racing inserts and erases: valid() (no key stored twice)");
        set_t::destroyDeviceObject(s);
    }

    // ---- part 3: churn until the table is full, then refusal exactly at max_size()
    {
        set_t s = set_t::createDeviceObject(32);
        s.set_excess_accounting(false); // keys until no slot is free, the reference's excess list aside
        const int max_size = s.max_size();
        std::vector<std::uint64_t> keys;
        for (int i = 0; i < 4 * max_size; ++i)
        {
            keys.push_back((rng() >> 4) + 7);
        }
        // insert and erase each block of max_size keys: every slot ends up erased
        for (int b = 0; b < 3; ++b)
        {
            std::vector<std::uint64_t> blk(keys.begin() + b * max_size, keys.begin() + (b + 1) * max_size);
            std::uint64_t* dk = to_device(blk);
            std::uint8_t* dok = nullptr;
            cudaMalloc(&dok, max_size);
            k_churn_set<<<(max_size + 255) / 256, 256>>>(s, dk, max_size, max_size, dok);
            const std::vector<std::uint8_t> ins = to_host(dok, max_size);
            k_churn_set<<<(max_size + 255) / 256, 256>>>(s, dk, 0, max_size, dok);
            cudaFree(dk);
            cudaFree(dok);
            int c = 0;
            for (auto x : ins)
            {
                c += x;
            }
            check(c == max_size, "fill: every key of a block of max_size() inserted (erased slots reused)");
        }
        std::vector<std::uint64_t> last(keys.begin() + 3 * max_size, keys.end());
        last.push_back(1);
        std::uint64_t* dk = to_device(last);
        std::uint8_t* dok = nullptr;
        cudaMalloc(&dok, last.size());
        k_churn_set<<<(static_cast<int>(last.size()) + 255) / 256, 256>>>(s, dk, static_cast<int>(last.size()),
                                                                     static_cast<int>(last.size()), dok);
        const std::vector<std::uint8_t> ok = to_host(dok, last.size());
        int c = 0;
        for (auto x : ok)
        {
            c += x;
        }
        check(c == max_size && s.size() == max_size, "full: max_size() keys stored, the one more refused");
        size_t stored = 0; // a key this launch did store
        while (stored + 1 < ok.size() && ok[stored] == 0)
        {
            ++stored;
        }
        std::vector<std::uint64_t> one(1, last[stored]);
        std::uint64_t* d1 = to_device(one);
        k_churn_set<<<1, 1>>>(s, d1, 0, 1, dok);     // erase one
        k_churn_set<<<1, 1>>>(s, d1 + 0, 1, 1, dok); // and insert it again into the slot it freed
        const std::vector<std::uint8_t> again = to_host(dok, 1);
        check(again[0] == 1 && s.size() == max_size && s.valid(), "full: an erase frees a slot the next insert takes");
        cudaFree(d1);
        cudaFree(dk);
        cudaFree(dok);
        set_t::destroyDeviceObject(s);
    }

    const cudaError_t e = cudaDeviceSynchronize();
    check(e == cudaSuccess, "no CUDA error");
    if (failures == 0)
    {
        std::printf("ALL PASS\n");
        return 0;
    }
    std::printf("%d FAILED\n", failures);
    return 1;
}

"""Large mixed workload plus containers (one GB300).

* unordered_map<uint64_t, uint32_t> with capacity 2^30 (max_size 1,752,476,107; 28 GB of slots),
  pre-filled with distinct keys to 0.5 / 0.75 / 0.9 x capacity, then interleaved insert / find batches
  of 2^24 keys each drawn Zipf(0.99) over a 2^34-rank universe;
* vector<uint32_t>::push_back of element i from 2^28 threads where mix(i) < 0.3 x 2^64;
* deque<uint64_t>: 2^26 mixed push_back / pop_front (50 / 50) on a deque half full;
* bitset::count over 2^33 bits at 50 % density.

Inputs are generated on the GPU with integer arithmetic that wraps mod 2^64.  Prefill keys are
i x (an odd constant) mod 2^61, a bijection, so they are distinct; Zipf keys carry bit 61, so the two
sets never meet.  Every part checks its own result with a
size-independent property.
"""

from __future__ import annotations

import torch

from . import containers as C

ODD_A = 0x9E3779B97F4A7C15 - (1 << 64)  # as int64
ODD_B = 0xBF58476D1CE4E5B9 - (1 << 64)
MASK61 = (1 << 61) - 1
BIT61 = 1 << 61


def lshr(x: torch.Tensor, k: int) -> torch.Tensor:
    """Logical right shift of int64 bits."""
    return (x >> k) & ((1 << (64 - k)) - 1)


def mix(x: torch.Tensor) -> torch.Tensor:
    """Bijective 64-bit mix on int64 bit patterns (xor-shift-multiply)."""
    z = x ^ lshr(x, 30)
    z = z * ODD_B
    z = z ^ lshr(z, 27)
    z = z * ODD_A
    return z ^ lshr(z, 31)


def zipf_keys(n: int, universe_log2: int, gen: torch.Generator, s: float = 0.99) -> torch.Tensor:
    u = torch.rand(n, dtype=torch.float64, device="cuda", generator=gen)
    a = 1.0 - s
    big = float(2 ** universe_log2)
    ranks = torch.floor((1.0 + u * (big ** a - 1.0)) ** (1.0 / a)).to(torch.int64)
    return (mix(ranks) & MASK61) | BIT61  # in [2^61, 2^62): never a reserved value, never a prefill key


def events():
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def timed(fn) -> float:
    a, b = events()
    torch.cuda.synchronize()
    a.record()
    fn()
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b)


def map_part(capacity_log2: int = 30, loads=(0.5, 0.75, 0.9), batch_log2: int = 24, rounds: int = 4) -> list:
    cap = 1 << capacity_log2
    gen = torch.Generator(device="cuda").manual_seed(2024)
    table = C.unordered_map.createDeviceObject(cap, key="u64", mapped="u32")
    out = []
    filled = 0
    expect = 0
    for load in loads:
        target = int(load * cap)
        # prefill with distinct keys below 2^61, value i
        chunk = 1 << 26
        t_fill = 0.0
        for lo in range(filled, target, chunk):
            hi = min(target, lo + chunk)
            idx = torch.arange(lo, hi, dtype=torch.int64, device="cuda")
            keys = (idx * ODD_A) & MASK61  # odd multiplier: a bijection of [0, 2^61)
            vals = idx.to(torch.int32)
            t_fill += timed(lambda: table.insert(keys, vals))
        expect += target - filled
        filled = target
        size0 = table.size()
        res = {"load": load, "prefill_keys": target, "size_after_prefill": size0, "expected_size": expect,
               "prefill_ms": t_fill}
        table.find(zipf_keys(1 << batch_log2, 34, gen))  # untimed: the first launch of a kernel loads its module
        ins_ms = find_ms = 0.0
        ins_keys = find_keys = 0
        ok = True
        for r in range(rounds):
            kins = zipf_keys(1 << batch_log2, 34, gen)
            before = table.size()
            present = table.contains(kins).bool()
            uniq_new = torch.unique(kins[~present]).numel()
            ins_ms += timed(lambda: table.insert(kins, (kins & 0xFFFFFFF).to(torch.int32)))
            ins_keys += kins.numel()
            ok = ok and table.size() == before + uniq_new
            kfind = zipf_keys(1 << batch_log2, 34, gen)
            holder = {}
            find_ms += timed(lambda: holder.update(r=table.find(kfind)))
            find_keys += kfind.numel()
            vals, found = holder["r"]
            # everything the insert batch stored is found with its value
            v2, f2 = table.find(kins)
            ok = ok and bool(f2.bool().all()) and bool(torch.equal(v2[present == 0], (kins[present == 0] & 0xFFFFFFF).to(torch.int32)))
        res.update({"insert_mops": ins_keys / (ins_ms * 1e-3) / 1e6, "find_mops": find_keys / (find_ms * 1e-3) / 1e6,
                    "batches": rounds, "batch_keys": 1 << batch_log2, "checks_pass": bool(ok and size0 == expect),
                    "final_size": table.size()})
        expect = res["final_size"]
        out.append(res)
    res_valid = table.valid()
    out.append({"valid": res_valid, "max_size": table.max_size()})
    C.unordered_base.destroyDeviceObject(table)
    return out


def vector_part(threads_log2: int = 28) -> dict:
    n = 1 << threads_log2
    idx = torch.arange(n, dtype=torch.int64, device="cuda")
    h = mix(idx)
    # mix(i) < 0.3 x 2^64 as unsigned: compare the top 62 bits
    thresh = int(0.3 * (1 << 62))
    pred = (lshr(h, 2) < thresh).to(torch.uint8)
    vals = idx.to(torch.int32)
    del h, idx
    v = C.vector.createDeviceObject(n, elem_bytes=4)
    v.push_back(vals[:1 << 16], pred[:1 << 16])  # untimed: loads the kernel's module
    v.clear()
    ms = timed(lambda: v.push_back(vals, pred))
    size = v.size()
    want = int(pred.sum())
    stored = v.data()
    ok = size == want and int(stored.to(torch.int64).sum()) == int(vals.to(torch.int64)[pred.bool()].sum())
    C.vector.destroyDeviceObject(v)
    return {"threads": n, "pushed": size, "expected": want, "ms": ms, "mpush_per_s": size / (ms * 1e-3) / 1e6,
            "checks_pass": bool(ok)}


def deque_part(ops_log2: int = 26) -> dict:
    n = 1 << ops_log2
    cap = 1 << (ops_log2 + 1)
    gen = torch.Generator(device="cuda").manual_seed(7)
    d = C.deque.createDeviceObject(cap, elem_bytes=8)
    init = torch.randint(0, 1 << 62, (cap // 2,), dtype=torch.int64, device="cuda", generator=gen)
    d.ops(None, init)
    warm = torch.zeros(1 << 12, dtype=torch.uint8, device="cuda")
    front, _ = d.ops(warm, init[: 1 << 12])  # untimed pops ...
    d.ops(None, front)  # ... and pushes of what they returned: the timed launch starts half full, same multiset
    is_push = (torch.rand(n, device="cuda", generator=gen) < 0.5).to(torch.uint8)
    vals = torch.randint(0, 1 << 62, (n,), dtype=torch.int64, device="cuda", generator=gen)
    holder = {}
    ms = timed(lambda: holder.update(r=d.ops(is_push, vals)))
    popped, ok = holder["r"]
    ip = is_push.bool()
    okb = ok.bool()
    rem = d.to_tensor()
    lhs = torch.sort(torch.cat([popped[~ip & okb], rem])).values
    rhs = torch.sort(torch.cat([init, vals[ip & okb]])).values
    good = bool(torch.equal(lhs, rhs)) and d.size() == cap // 2 + int((ip & okb).sum()) - int((~ip & okb).sum())
    C.deque.destroyDeviceObject(d)
    return {"ops": n, "capacity": cap, "ms": ms, "mops": n / (ms * 1e-3) / 1e6, "succeeded": int(okb.sum()),
            "checks_pass": good}


def bitset_part(bits_log2: int = 33) -> dict:
    nwords = 1 << (bits_log2 - 5)
    gen = torch.Generator(device="cuda").manual_seed(3)
    words = torch.randint(-(2**31), 2**31, (nwords,), dtype=torch.int32, device="cuda", generator=gen)
    C.bitset_count(words, nwords * 32)  # warm-up
    holder = {}
    ms = timed(lambda: holder.update(c=C.bitset_count(words, nwords * 32)))
    x = words.to(torch.int64) & 0xFFFFFFFF
    cnt = torch.zeros((), dtype=torch.int64, device="cuda")
    for b in range(32):
        cnt += ((x >> b) & 1).sum()
    good = holder["c"] == int(cnt)
    return {"bits": nwords * 32, "count": holder["c"], "ms": ms, "gb_per_s": nwords * 4 / (ms * 1e-3) / 1e9,
            "checks_pass": bool(good)}


def run(full: bool = True) -> dict:
    if full:
        m = map_part()
        return {"map": m, "vector": vector_part(), "deque": deque_part(), "bitset": bitset_part()}
    return {"map": map_part(capacity_log2=22, batch_log2=18, rounds=2), "vector": vector_part(22),
            "deque": deque_part(20), "bitset": bitset_part(26)}


if __name__ == "__main__":
    # one part at a chosen size, e.g. for a profiler capture of its kernel:
    #   python -m stdgpu_gb300.large_bench --part bitset --log2 31
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("--part", choices=["map", "vector", "deque", "bitset"], required=True)
    ap.add_argument("--log2", type=int, required=True,
                    help="map: capacity; vector: threads; deque: operations; bitset: bits (log2)")
    a = ap.parse_args()
    if a.part == "map":
        r = map_part(capacity_log2=a.log2, batch_log2=max(10, a.log2 - 6), rounds=2)
    elif a.part == "vector":
        r = vector_part(a.log2)
    elif a.part == "deque":
        r = deque_part(a.log2)
    else:
        r = bitset_part(a.log2)
    print(json.dumps(r))

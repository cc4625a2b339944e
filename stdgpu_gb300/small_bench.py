"""Small-table workload: unordered_set<uint32_t>, capacity 2^21, 2^20 keys (one GB300).

The table (3.4 M slots x 4 B = 13.7 MB) lives in L2, so the kernels are short and a step is bound by
launch overhead as much as by memory.  Keys are uniform in [0, 2^32 - 2] (seeded); contains queries
alternate inserted keys and fresh ones; erase takes a random half of the keys.  One step = clear +
insert + contains + erase, timed eagerly (four launches) and as one replayed CUDA graph.
"""

from __future__ import annotations

from ctypes import c_void_p

import numpy as np
import torch

from . import _native as N
from . import containers as C


def make_inputs(n: int = 1 << 20, seed: int = 0):
    rng = np.random.default_rng(seed)
    keys = rng.integers(0, 2**32 - 1, size=n, dtype=np.uint64).astype(np.uint32)
    fresh = rng.integers(0, 2**32 - 1, size=n, dtype=np.uint64).astype(np.uint32)
    queries = np.where(np.arange(n) % 2 == 0, keys[rng.integers(0, n, size=n)], fresh)
    erase = keys[rng.permutation(n)[: n // 2]]
    return keys, queries, erase


def run(steps: int = 20, warmup: int = 5, capacity: int = 1 << 21, n: int = 1 << 20) -> dict:
    keys_np, queries_np, erase_np = make_inputs(n)
    dev = lambda a: torch.from_numpy(a.view(np.int32).copy()).cuda()
    keys, queries, erase = dev(keys_np), dev(queries_np), dev(erase_np)
    flags = torch.empty(n, dtype=torch.uint8, device="cuda")
    t = C.unordered_set.createDeviceObject(capacity, key="u32")
    lib = N.load()
    stream = torch.cuda.Stream()
    sp = c_void_p(stream.cuda_stream)
    h = t._h

    def step():
        N.check(lib.sg_unordered_clear(h, sp), "clear")
        N.check(lib.sg_unordered_insert_kv(h, c_void_p(keys.data_ptr()), None, n, None, sp), "insert")
        N.check(lib.sg_unordered_contains(h, c_void_p(queries.data_ptr()), n, c_void_p(flags.data_ptr()), sp),
                "contains")
        N.check(lib.sg_unordered_erase(h, c_void_p(erase.data_ptr()), len(erase_np), None, sp), "erase")

    def timed(fn):
        with torch.cuda.stream(stream):
            for _ in range(warmup):
                fn()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(steps):
                fn()
            b.record(stream)
        stream.synchronize()
        return a.elapsed_time(b) / steps

    eager_ms = timed(step)
    distinct = len(np.unique(keys_np))
    erased = len(np.intersect1d(np.unique(erase_np), np.unique(keys_np)))
    ok = t.size(stream) == distinct - erased
    hits = int(flags.sum().item())
    want_hits = int(np.isin(queries_np, keys_np).sum())
    ok = ok and hits == want_hits
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph, stream=stream):
        step()
    graph_ms = timed(graph.replay)
    ok = ok and t.size(stream) == distinct - erased and int(flags.sum().item()) == want_hits
    table_bytes = (t.geometry().num_groups + 1) * 128
    C.unordered_base.destroyDeviceObject(t)
    ops = n + n + len(erase_np)
    return {"keys": n, "capacity": capacity, "table_bytes": table_bytes,
            "eager_ms": eager_ms, "graph_ms": graph_ms, "eager_mops": ops / (eager_ms * 1e-3) / 1e6,
            "graph_mops": ops / (graph_ms * 1e-3) / 1e6, "checks_pass": bool(ok)}

"""Many-small-tables workload: 4096 unordered_set<uint64_t> with lognormal key counts.

Per-table key counts are lognormal (median 2048, sigma 1.5, clipped to 64..262144); capacity is
2 x count rounded up to a power of two; keys are uniform uint64 (seed = table id); contains queries
are half stored keys, half fresh.  One step = clear + insert + contains over every table, run three
ways on the same GB300:

* plain:   one createDeviceObject per table, then 3 calls per table per step (clear, insert, contains),
           issued from a C++ loop over the C ABI
* batched: one batch object, 3 batched calls per step (each one persistent launch plus a tile count)
* graph:   the batched step captured once in a CUDA graph and replayed

Used by bench.py (--workload batched) and by autotune.py.
"""

from __future__ import annotations

import time
from ctypes import c_void_p

import numpy as np
import torch

from . import comparators as P
from . import containers as C
from . import workloads as W


def make_workload(n_tables: int = 4096, seed: int = 0):
    counts = W.lognormal_counts(n_tables, seed=seed)
    caps = np.array([1 << int(np.ceil(np.log2(2 * c))) for c in counts], dtype=np.int64)
    keys = [W.table_keys_u64(t, int(c)) for t, c in enumerate(counts)]
    rng = np.random.default_rng(seed + 7)
    queries = []
    for t, c in enumerate(counts):
        hit = keys[t][rng.integers(0, c, size=c)]
        fresh = rng.integers(0, 2**64 - 1, size=c, dtype=np.uint64)
        queries.append(np.where(np.arange(c) % 2 == 0, hit, fresh))
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    return counts, caps, np.concatenate(keys), np.concatenate(queries), offsets


def to_dev(a: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).cuda()


def time_batched(batch: C.table_batch, d_keys, d_q, d_off, out, steps: int, warmup: int) -> float:
    st = torch.cuda.current_stream()
    for _ in range(warmup):
        batch.clear(stream=st)
        batch.insert(d_keys, d_off, stream=st)
        batch.contains(d_q, d_off, out=out, stream=st)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    a.record(st)
    for _ in range(steps):
        batch.clear(stream=st)
        batch.insert(d_keys, d_off, stream=st)
        batch.contains(d_q, d_off, out=out, stream=st)
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def time_graph(batch: C.table_batch, d_keys, d_q, d_off, out, steps: int, warmup: int) -> float:
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(2):
            batch.clear(stream=s)
            batch.insert(d_keys, d_off, stream=s)
            batch.contains(d_q, d_off, out=out, stream=s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        st = torch.cuda.current_stream()
        batch.clear(stream=st)
        batch.insert(d_keys, d_off, stream=st)
        batch.contains(d_q, d_off, out=out, stream=st)
    for _ in range(warmup):
        g.replay()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    a.record(st)
    for _ in range(steps):
        g.replay()
    b.record(st)
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def time_plain(caps, d_keys, d_q, offsets, out, steps: int, warmup: int) -> tuple[float, float]:
    """Plain per-table C-ABI calls (clear, insert, contains per table) on the current stream, from a C++ loop
    (comparators.plain_tables_steps).  Returns (GPU ms per step, host ms per step)."""
    tables = [C.unordered_set.createDeviceObject(int(c), key="u64") for c in caps]
    for t in tables:
        t.set_excess_accounting(False)  # the batched object's semantics: keys until no slot is free
    st = torch.cuda.current_stream()
    P.plain_tables_steps(tables, d_keys, d_q, offsets, 8, out, warmup, st)
    gpu_ms, host_ms = P.plain_tables_steps(tables, d_keys, d_q, offsets, 8, out, steps, st)
    for t in tables:
        C.unordered_base.destroyDeviceObject(t)
    return gpu_ms, host_ms


def run(steps: int = 5, warmup: int = 3, tuning: dict | None = None) -> dict:
    counts, caps, keys, queries, offsets = make_workload()
    d_keys, d_q, d_off = to_dev(keys), to_dev(queries), to_dev(offsets)
    out = torch.zeros(len(queries), dtype=torch.uint8, device="cuda")
    batch = C.table_batch.createDeviceObjects(caps, key="u64", tuning=tuning)
    batched_ms = time_batched(batch, d_keys, d_q, d_off, out, steps, warmup)
    hits = int(out.sum())
    sizes = batch.sizes()
    graph_ms = time_graph(batch, d_keys, d_q, d_off, out, steps, warmup)
    hits_graph = int(out.sum())
    storage = batch.storage_bytes()
    C.table_batch.destroyDeviceObjects(batch)
    plain_ms, plain_host_ms = time_plain(caps, d_keys, d_q, offsets, out, max(1, steps // 2), 1)
    hits_plain = int(out.sum())
    expect = np.array([len(np.unique(keys[offsets[t]:offsets[t + 1]])) for t in range(len(counts))])
    ops = int(counts.sum()) * 2
    return {
        "tables": len(counts), "keys": int(counts.sum()), "queries": int(counts.sum()),
        "storage_bytes": storage,
        "batched_ms": batched_ms, "graph_ms": graph_ms, "plain_ms": plain_ms, "plain_host_ms": plain_host_ms,
        "speedup_batched": plain_ms / batched_ms, "speedup_graph": plain_ms / graph_ms,
        "batched_mops": ops / (batched_ms * 1e-3) / 1e6, "graph_mops": ops / (graph_ms * 1e-3) / 1e6,
        "plain_mops": ops / (plain_ms * 1e-3) / 1e6,
        "results_agree": bool(hits == hits_graph == hits_plain and np.array_equal(sizes, expect)),
        "launches_per_step": {"plain": 3 * len(counts), "batched": 5},
    }

"""Batched many-table objects against the oracle restatement, table by table, and under CUDA-graph replay."""

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import workloads as W

from gpu_util import dev, host, per_key_success

pytestmark = pytest.mark.gpu


def make_case(kind, n_tables, seed, max_n=3000):
    rng = np.random.default_rng(seed)
    counts = rng.integers(0, max_n, size=n_tables)
    counts[::7] = 0  # some empty tables
    counts[1] = 1
    kd, vd = O.KEY_DTYPE[kind], O.VAL_DTYPE[kind]
    hi = 2**32 - 1 if kd == np.uint32 else 2**64 - 1
    keys = []
    for t, c in enumerate(counts):
        k = rng.integers(0, hi, size=c, dtype=np.uint64)
        if c > 4:
            k[: c // 4] = k[c // 4: 2 * (c // 4)]  # duplicates inside a table
        keys.append(k.astype(kd))
    offsets = np.concatenate([[0], np.cumsum(counts)]).astype(np.int64)
    caps = np.maximum(1, 2 * counts).astype(np.int64)
    flat = np.concatenate(keys) if len(keys) else np.zeros(0, kd)
    vals = (W.mix64(flat.astype(np.uint64)) & np.uint64(0xFFFFFFFF)).astype(vd) if vd is not None else None
    return counts, offsets, caps, keys, flat, vals


@pytest.mark.parametrize("kind", [O.SET_U64, O.MAP_U64_U32, O.SET_U32, O.MAP_U64_U64])
def test_batch_matches_oracle_per_table(kind):
    counts, offsets, caps, keys, flat, vals = make_case(kind, 97, seed=kind)
    kd, vd = O.KEY_DTYPE[kind], O.VAL_DTYPE[kind]
    key_s = "u32" if kd == np.uint32 else "u64"
    mapped_s = None if vd is None else ("u32" if vd == np.uint32 else "u64")
    b = sg.table_batch.createDeviceObjects(caps, key=key_s, mapped=mapped_s)
    d_off = dev(offsets)
    flags = torch.zeros(len(flat), dtype=torch.uint8, device="cuda")
    b.insert(dev(flat), d_off, dev(vals) if vals is not None else None, flags=flags)
    f = flags.cpu().numpy()
    sizes = b.sizes()
    ports = []
    for t in range(len(counts)):
        P = O.PortTable(kind, int(caps[t]))
        lo, hi_ = offsets[t], offsets[t + 1]
        pf = P.insert(flat[lo:hi_], vals[lo:hi_] if vals is not None else None, flags=True)
        assert per_key_success(flat[lo:hi_], f[lo:hi_]) == per_key_success(flat[lo:hi_], pf), t
        assert sizes[t] == P.size(), t
        ports.append(P)
    # queries: half stored keys, half fresh, per table
    rng = np.random.default_rng(99)
    q = []
    for t in range(len(counts)):
        c = counts[t]
        stored = keys[t][rng.integers(0, c, size=c)] if c else np.zeros(0, kd)
        fresh = rng.integers(0, 2**31, size=c, dtype=np.uint64).astype(kd)
        q.append(np.where(rng.random(c) < 0.5, stored, fresh).astype(kd))
    qflat = np.concatenate(q)
    vals_g, found = b.find(dev(qflat), d_off)
    found = found.cpu().numpy()
    cont = b.contains(dev(qflat), d_off).cpu().numpy()
    assert np.array_equal(found, cont)
    for t in range(len(counts)):
        lo, hi_ = offsets[t], offsets[t + 1]
        pv, pf = ports[t].find(q[t])
        assert np.array_equal(found[lo:hi_], pf), t
        if vd is not None:
            gv = host(vals_g, vd)[lo:hi_]
            assert np.array_equal(gv[pf == 1], pv[pf == 1]), t
    # erase half the stored keys of each table
    e = [keys[t][: counts[t] // 2] for t in range(len(counts))]
    eflat = np.concatenate(e)
    eoff = np.concatenate([[0], np.cumsum([len(x) for x in e])]).astype(np.int64)
    ef = torch.zeros(len(eflat), dtype=torch.uint8, device="cuda")
    b.erase(dev(eflat), dev(eoff), flags=ef)
    ef = ef.cpu().numpy()
    sizes = b.sizes()
    for t in range(len(counts)):
        pe = ports[t].erase(e[t], flags=True)
        assert per_key_success(e[t], ef[eoff[t]:eoff[t + 1]]) == per_key_success(e[t], pe), t
        assert sizes[t] == ports[t].size(), t
    sg.table_batch.destroyDeviceObjects(b)


def test_batch_equals_single_table_path_and_views_are_valid():
    counts, offsets, caps, keys, flat, _ = make_case(O.SET_U64, 40, seed=5)
    b = sg.table_batch.createDeviceObjects(caps, key="u64")
    d_off = dev(offsets)
    b.insert(dev(flat), d_off)
    got = b.contains(dev(flat), d_off).cpu().numpy()
    assert got.sum() == len(flat)
    for t in range(len(counts)):
        s = sg.unordered_set.createDeviceObject(int(caps[t]), key="u64")
        if counts[t]:
            s.insert(dev(keys[t]))
        assert s.size() == b.sizes()[t]
        # the batched table's geometry equals a single table's
        v = b.view(t)
        assert v.total_count == s.max_size() and v.bucket_count == s.bucket_count()
        sg.unordered_base.destroyDeviceObject(s)
    sg.table_batch.destroyDeviceObjects(b)


@pytest.mark.parametrize("threads,bpsm,tiles", [(128, 2, 1), (256, 0, 4), (512, 1, 2)])
def test_batch_launch_shapes_give_same_results(threads, bpsm, tiles):
    counts, offsets, caps, keys, flat, _ = make_case(O.SET_U64, 200, seed=7)
    b = sg.table_batch.createDeviceObjects(caps, key="u64", tuning={"threads_per_block": threads,
                                                                   "blocks_per_sm": bpsm, "tiles_per_step": tiles})
    d_off = dev(offsets)
    b.insert(dev(flat), d_off)
    sizes = b.sizes()
    expect = np.array([len(np.unique(k)) for k in keys])
    assert np.array_equal(sizes, expect)
    assert b.contains(dev(flat), d_off).cpu().numpy().sum() == len(flat)
    sg.table_batch.destroyDeviceObjects(b)


def test_batch_cuda_graph_replay():
    """clear + insert + contains captured once, replayed: identical results every replay."""
    counts, offsets, caps, keys, flat, _ = make_case(O.SET_U64, 300, seed=11)
    b = sg.table_batch.createDeviceObjects(caps, key="u64")
    d_keys = dev(flat)
    d_off = dev(offsets)
    out = torch.zeros(len(flat), dtype=torch.uint8, device="cuda")
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(s):
        for _ in range(2):  # warm-up outside capture
            b.clear(stream=s)
            b.insert(d_keys, d_off, stream=s)
            b.contains(d_keys, d_off, out=out, stream=s)
    torch.cuda.current_stream().wait_stream(s)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        st = torch.cuda.current_stream()
        b.clear(stream=st)
        b.insert(d_keys, d_off, stream=st)
        b.contains(d_keys, d_off, out=out, stream=st)
    expect = np.array([len(np.unique(k)) for k in keys])
    for _ in range(3):
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        assert out.cpu().numpy().sum() == len(flat)
        assert np.array_equal(b.sizes(), expect)
    sg.table_batch.destroyDeviceObjects(b)

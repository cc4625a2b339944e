"""Parity on the benchmark configurations' own shapes.

* voxel map (unordered_map<uint64_t,uint32_t>, capacity 2^28, 2^27 keys): the benchmark's exact call
  sequence -- clear, insert of value_type pairs with no flags (the partitioned path), find, erase (the
  partitioned path) -- with every result checked element by element; at 2^20 keys the same step against
  the oracle restatement.
* 4096 lognormal-sized unordered_set<uint64_t> in one batch object: per-key insert outcomes, contains
  answers, erase outcomes and sizes against one oracle table per set.
* the large mixed map at a reduced capacity (2^22): pre-fill to 0.5 / 0.75 / 0.9 load, then Zipf(0.99)
  insert and find batches, per-key outcomes, values and sizes against the oracle.
"""

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import batch_bench, large_bench
from stdgpu_gb300.voxel_step import VoxelStep

from gpu_util import dev, host, per_key_success

pytestmark = pytest.mark.gpu


def test_voxel_step_full_size_element_by_element():
    """2^27 keys into capacity 2^28: insert and erase take the partitioned path (three launches each:
    scatter, ordered kernel, gated direct kernel); sizes after every call, all 2^27 found flags and values,
    and the 2^27 - 2^25 remaining elements with their values are checked; a second step on the cleared
    table gives the same."""
    vs = VoxelStep(27, torch.device("cuda", 0))
    st = torch.cuda.current_stream()
    try:
        for _ in range(2):
            seen = vs.checked_step(st)
            assert seen["insert_launches"] == 3, seen
            assert seen["erase_launches"] == 3, seen
            assert seen["checked_elements"] == (1 << 27) - (1 << 25)
        assert vs.table.valid()
    finally:
        vs.close()


def test_voxel_step_small_against_oracle():
    """The same step at 2^20 keys (direct kernels at this size) and in partitioned mode, against the oracle
    restatement: find answers and values, size, final contents."""
    for mode in ("auto", "partitioned"):
        vs = VoxelStep(20, torch.device("cuda", 0))
        vs.table.set_insert_mode(mode)
        st = torch.cuda.current_stream()
        try:
            vs.checked_step(st)
            w = vs.w
            P = O.PortTable(O.MAP_U64_U32, vs.capacity)
            P.insert(w.keys, w.values)
            pv, pf = P.find(w.queries)
            P.erase(w.erase)
            gf = vs.out_found.cpu().numpy()
            gv = host(vs.out_vals, np.uint32)
            assert np.array_equal(gf, pf)
            assert np.array_equal(gv[pf == 1], pv[pf == 1])
            assert vs.table.size() == P.size()
            pk, pvals = P.range()
            o = np.argsort(pk)
            gk, gvals = vs.table.range_copy()
            gk, gvals = host(gk, np.uint64), host(gvals, np.uint32)
            og = np.argsort(gk)
            assert np.array_equal(gk[og], pk[o]) and np.array_equal(gvals[og], pvals[o])
            P.close()
        finally:
            vs.close()


def test_batched_4096_lognormal_tables_against_oracle():
    """The batched configuration itself: 4096 sets with lognormal counts (median 2048, sigma 1.5, clipped to
    64..262144; 24.6 M keys), capacity bit_ceil(2 count); a table of up to 262,144 keys spans many work-list
    tiles.  Every 5th key is replaced by an earlier key of its table so duplicates race.  Per-key insert
    outcomes, contains answers (50 % hits), per-key erase outcomes and sizes equal one oracle table per set."""
    counts, caps, keys, queries, offsets = batch_bench.make_workload(4096, seed=0)
    for t in range(len(counts)):
        lo, hi = offsets[t], offsets[t + 1]
        seg = keys[lo:hi]
        seg[5::5] = seg[: len(seg[5::5])]
    b = sg.table_batch.createDeviceObjects(caps, key="u64")
    d_off = dev(offsets)
    flags = torch.zeros(len(keys), dtype=torch.uint8, device="cuda")
    b.insert(dev(keys), d_off, flags=flags)
    f = flags.cpu().numpy()
    cont = b.contains(dev(queries), d_off).cpu().numpy()
    # erase: the first half of each table's keys plus a few absent ones
    er, eoff = [], [0]
    for t in range(len(counts)):
        lo, hi = offsets[t], offsets[t + 1]
        e = np.concatenate([keys[lo: lo + (hi - lo) // 2], queries[lo + 1: hi: 7]])
        er.append(e)
        eoff.append(eoff[-1] + len(e))
    eflat = np.concatenate(er)
    eoff = np.array(eoff, np.int64)
    ef = torch.zeros(len(eflat), dtype=torch.uint8, device="cuda")
    sizes_ins = b.sizes()
    b.erase(dev(eflat), dev(eoff), flags=ef)
    ef = ef.cpu().numpy()
    sizes_er = b.sizes()
    cont2 = b.contains(dev(queries), d_off).cpu().numpy()
    bad = []
    for t in range(len(counts)):
        lo, hi = offsets[t], offsets[t + 1]
        P = O.PortTable(O.SET_U64, int(caps[t]))
        pf = P.insert(keys[lo:hi], flags=True)
        if per_key_success(keys[lo:hi], f[lo:hi]) != per_key_success(keys[lo:hi], pf) or sizes_ins[t] != P.size():
            bad.append((t, "insert"))
        if not np.array_equal(cont[lo:hi], P.contains(queries[lo:hi])):
            bad.append((t, "contains"))
        pe = P.erase(er[t], flags=True)
        if per_key_success(er[t], ef[eoff[t]:eoff[t + 1]]) != per_key_success(er[t], pe) or sizes_er[t] != P.size():
            bad.append((t, "erase"))
        if not np.array_equal(cont2[lo:hi], P.contains(queries[lo:hi])):
            bad.append((t, "contains after erase"))
        P.close()
    sg.table_batch.destroyDeviceObjects(b)
    assert not bad, bad[:10]


def test_large_map_zipf_batches_against_oracle():
    """unordered_map<uint64_t,uint32_t> of capacity 2^22, pre-filled with distinct keys to 0.5, 0.75 and 0.9
    load, each followed by two Zipf(0.99) insert batches (2^18 keys over 2^34 ranks, many repeats; value a
    function of the key) and two Zipf find batches, as the large workload runs them at capacity 2^30:
    per-key insert outcomes, sizes, find answers and values equal the oracle's."""
    cap = 1 << 22
    t = sg.unordered_map.createDeviceObject(cap, key="u64", mapped="u32")
    P = O.PortTable(O.MAP_U64_U32, cap)
    gen = torch.Generator(device="cuda").manual_seed(2024)
    filled = 0
    try:
        for load in (0.5, 0.75, 0.9):
            target = int(load * cap)
            idx = torch.arange(filled, target, dtype=torch.int64, device="cuda")
            pk = (idx * large_bench.ODD_A) & large_bench.MASK61
            pv = idx.to(torch.int32)
            before = P.size()
            t.insert(pk, pv)
            P.insert(host(pk, np.uint64), host(pv, np.uint32))
            # pre-fill keys are distinct and below 2^61, Zipf keys carry bit 61: every pre-fill key is new
            assert t.size() == P.size() == before + (target - filled)
            filled = target
            for _ in range(2):
                kins = large_bench.zipf_keys(1 << 18, 34, gen)
                vins = (kins & 0xFFFFFFF).to(torch.int32)
                fl = torch.zeros(kins.numel(), dtype=torch.uint8, device="cuda")
                t.insert(kins, vins, flags=fl)
                hk = host(kins, np.uint64)
                pf = P.insert(hk, host(vins, np.uint32), flags=True)
                assert per_key_success(hk, fl.cpu().numpy()) == per_key_success(hk, pf)
                assert t.size() == P.size()
                kf = large_bench.zipf_keys(1 << 18, 34, gen)
                gv, gf = t.find(kf)
                hv, hf = P.find(host(kf, np.uint64))
                gf = gf.cpu().numpy()
                assert np.array_equal(gf, hf)
                assert np.array_equal(host(gv, np.uint32)[hf == 1], hv[hf == 1])
        assert t.valid()
    finally:
        sg.unordered_base.destroyDeviceObject(t)
        P.close()

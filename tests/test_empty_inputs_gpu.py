"""Empty and degenerate inputs on every bulk entry point (the reference's tests call each bulk operation
with empty ranges, tests/stdgpu/unordered_datastructure.inc): nothing changes, nothing fails."""

import numpy as np
import pytest
import torch

import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

from gpu_util import dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("key,mapped", [("u32", None), ("u64", None), ("u64", "u32"), ("u64", "u64"),
                                        ("u32", "u32"), ("u32", "u64")])
def test_table_calls_on_empty_ranges(key, mapped):
    t = (sg.unordered_set.createDeviceObject(1000, key=key) if mapped is None
         else sg.unordered_map.createDeviceObject(1000, key=key, mapped=mapped))
    kd = torch.int32 if key == "u32" else torch.int64
    md = None if mapped is None else (torch.int32 if mapped == "u32" else torch.int64)
    empty_k = torch.empty(0, dtype=kd, device="cuda")
    empty_m = None if md is None else torch.empty(0, dtype=md, device="cuda")
    for mode in ("direct", "partitioned"):
        t.set_insert_mode(mode)
        t.insert(empty_k, empty_m)
        t.erase(empty_k)
    vals, found = t.find(empty_k)
    assert found.numel() == 0
    assert t.contains(empty_k).numel() == 0
    assert t.size() == 0 and t.empty() and t.valid()
    assert t.device_range().numel() == 0
    k, v = t.range_copy()
    assert k.numel() == 0
    t.rehash(2000)
    assert t.size() == 0 and t.valid()
    sg.unordered_base.destroyDeviceObject(t)


def test_containers_on_empty_inputs():
    v = sg.vector.createDeviceObject(10, elem_bytes=4)
    v.push_back(torch.empty(0, dtype=torch.int32, device="cuda"))
    v.insert(torch.empty(0, dtype=torch.int32, device="cuda"))
    v.erase(0)
    vals, ok = v.pop_back(0)
    assert v.size() == 0 and ok.numel() == 0
    vals, ok = v.pop_back(3)  # popping an empty vector fails for every element
    assert int(ok.sum()) == 0 and v.size() == 0
    sg.vector.destroyDeviceObject(v)
    d = sg.deque.createDeviceObject(10, elem_bytes=8)
    assert d.push_back(torch.empty(0, dtype=torch.int64, device="cuda")).numel() == 0
    assert d.push_front(torch.empty(0, dtype=torch.int64, device="cuda")).numel() == 0
    for pop in (d.pop_front, d.pop_back):
        vals, ok = pop(4)
        assert int(ok.sum()) == 0
    assert d.size() == 0 and d.to_tensor().numel() == 0
    sg.deque.destroyDeviceObject(d)
    assert sg.bitset_count(torch.zeros(1, dtype=torch.int32, device="cuda"), 0) == 0


def test_batch_of_empty_tables():
    """All ranges empty: an empty key tensor (a NULL pointer) walks no tile."""
    b = sg.table_batch.createDeviceObjects([1, 100, 1000], key="u64")
    offsets = torch.zeros(4, dtype=torch.int64, device="cuda")
    keys = torch.empty(0, dtype=torch.int64, device="cuda")
    b.insert(keys, offsets)
    assert b.contains(keys, offsets).numel() == 0
    assert list(b.sizes()) == [0, 0, 0]
    sg.table_batch.destroyDeviceObjects(b)

"""Table calls on host buffers (sg_*_host through a stager) against the same calls on device buffers and
against the oracle: chunking, ring wrap, ragged last chunk, empty calls, pageable memory, and stream order."""

from ctypes import c_void_p

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

from gpu_util import dev, host, per_key_success

pytestmark = pytest.mark.gpu


def pinned(a: np.ndarray) -> torch.Tensor:
    v = {4: np.int32, 8: np.int64, 1: np.uint8}[a.dtype.itemsize]
    return torch.from_numpy(np.ascontiguousarray(a).view(v).copy()).pin_memory()


def cpu(a: np.ndarray) -> torch.Tensor:
    v = {4: np.int32, 8: np.int64, 1: np.uint8}[a.dtype.itemsize]
    return torch.from_numpy(np.ascontiguousarray(a).view(v).copy())


@pytest.mark.parametrize("chunk,buffers,ready", [(1000, 2, False), (4096, 3, False), (1 << 20, 4, False),
                                                  (1000, 2, True), (4096, 3, True)])
def test_map_host_calls_match_oracle(chunk, buffers, ready):
    """With inputs declared ready the uploads of a call overlap the previous call's kernels; the results are
    the same."""
    rng = np.random.default_rng(chunk)
    n = 50_000 + 123  # ragged last chunk
    keys = rng.integers(0, 2**63, size=n, dtype=np.uint64)
    keys[::7] = keys[::5][: len(keys[::7])]  # duplicates inside one call
    vals = rng.integers(0, 2**32, size=n, dtype=np.uint64).astype(np.uint32)
    st = sg.stager(chunk, buffers)
    st.set_inputs_ready(ready)
    t = sg.unordered_map.createDeviceObject(1 << 17, key="u64", mapped="u32")
    port = O.PortTable(O.MAP_U64_U32, 1 << 17)
    flags = torch.zeros(n, dtype=torch.uint8).pin_memory()
    t.insert(pinned(keys), pinned(vals), flags=flags, stager=st)
    want = port.insert(keys, vals, flags=True)
    assert per_key_success(keys, flags.numpy()) == per_key_success(keys, want)
    assert t.size() == port.size()
    q = np.concatenate([keys[:20000], rng.integers(0, 2**63, size=9000, dtype=np.uint64)])
    gv, gf = t.find(pinned(q), stager=st)
    pv, pf = port.find(q)
    assert np.array_equal(gf.numpy(), pf)
    # values of present keys: any inserted copy's value is allowed for duplicates, so compare with the
    # device path on the same table
    dv, df = t.find(dev(q))
    assert np.array_equal(gv.numpy().view(np.uint32)[pf == 1], host(dv, np.uint32)[pf == 1])
    assert np.all(gv.numpy()[pf == 0] == 0)
    assert np.array_equal(t.contains(pinned(q), stager=st).numpy(), pf)
    er = keys[:30000:3]
    eflags = torch.zeros(len(er), dtype=torch.uint8).pin_memory()
    t.erase(pinned(er), flags=eflags, stager=st)
    want_e = port.erase(er, flags=True)
    assert per_key_success(er, eflags.numpy()) == per_key_success(er, want_e)
    assert t.size() == port.size()
    assert t.valid()
    sg.unordered_base.destroyDeviceObject(t)
    st.close()


def test_set_u32_pageable_and_empty():
    rng = np.random.default_rng(3)
    keys = rng.integers(0, 2**32, size=20000, dtype=np.uint64).astype(np.uint32)
    st = sg.stager(3000, 2)
    t = sg.unordered_set.createDeviceObject(1 << 15, key="u32")
    port = O.PortTable(O.SET_U32, 1 << 15)
    t.insert(cpu(keys), stager=st)  # pageable host memory
    port.insert(keys)
    assert t.size() == port.size()
    assert np.array_equal(t.contains(cpu(keys[::2]), stager=st).numpy(), port.contains(keys[::2]))
    empty = torch.empty(0, dtype=torch.int32)
    t.insert(empty, stager=st)
    t.erase(empty, stager=st)
    assert t.contains(empty, stager=st).numel() == 0
    assert t.size() == port.size()
    sg.unordered_base.destroyDeviceObject(t)
    st.close()


def test_host_calls_are_stream_ordered_without_sync():
    """insert_host, then a device-pointer find queued right behind it on the same stream, then
    find_host into pinned outputs: one synchronisation at the end sees every result."""
    lib = sg.load()
    rng = np.random.default_rng(9)
    n = 300_000
    keys = np.unique(rng.integers(0, 2**62, size=n, dtype=np.uint64))
    n = len(keys)
    pairs = np.zeros((n, 2), np.uint64)
    pairs[:, 0] = keys
    pairs[:, 1] = np.arange(n, dtype=np.uint64)
    pairs_h = pinned(pairs.reshape(-1))
    keys_h = pinned(keys)
    vals_h = torch.zeros(n, dtype=torch.int32).pin_memory()
    found_h = torch.zeros(n, dtype=torch.uint8).pin_memory()
    keys_d = dev(keys)
    found_d = torch.zeros(n, dtype=torch.uint8, device="cuda")
    st = sg.stager(1 << 15, 3)
    t = sg.unordered_map.createDeviceObject(1 << 19, key="u64", mapped="u32")
    s = torch.cuda.Stream()
    sp = c_void_p(s.cuda_stream)
    torch.cuda.synchronize()
    assert lib.sg_unordered_insert_host(t._h, st._h, c_void_p(pairs_h.data_ptr()), n, None, sp) == 0
    assert lib.sg_unordered_contains(t._h, c_void_p(keys_d.data_ptr()), n, c_void_p(found_d.data_ptr()), sp) == 0
    assert lib.sg_unordered_find_host(t._h, st._h, c_void_p(keys_h.data_ptr()), n, c_void_p(vals_h.data_ptr()),
                                      c_void_p(found_h.data_ptr()), sp) == 0
    s.synchronize()
    assert int(found_d.sum()) == n
    assert int(found_h.sum()) == n
    assert np.array_equal(vals_h.numpy().view(np.uint32), np.arange(n, dtype=np.uint32))
    sg.unordered_base.destroyDeviceObject(t)
    st.close()


def test_stager_rejects_bad_arguments():
    lib = sg.load()
    h = c_void_p()
    from ctypes import byref
    assert lib.sg_stager_create(0, 4, byref(h)) == N.SG_ERR_BAD_ARG
    assert lib.sg_stager_create(1024, 1, byref(h)) == N.SG_ERR_BAD_ARG
    assert lib.sg_stager_create(1024, 9, byref(h)) == N.SG_ERR_BAD_ARG
    assert lib.sg_stager_create((1 << 30) + 1, 4, byref(h)) == N.SG_ERR_BAD_ARG

"""Snapshots and rehash on the GPU: a loaded table is bit for bit the saved one (same slots, same answers,
erased slots and out-of-band keys included); rehash into a larger or smaller capacity keeps every element,
and refuses, leaving the table unchanged, when they do not fit."""

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

from gpu_util import dev, host

pytestmark = pytest.mark.gpu


def filled_map(rng, cap=1 << 16, n=40000):
    t = sg.unordered_map.createDeviceObject(cap, key="u64", mapped="u64")
    keys = rng.integers(0, 2**64 - 1, size=n, dtype=np.uint64)
    keys[:2] = [2**64 - 1, 2**64 - 2]  # the out-of-band values
    vals = keys ^ np.uint64(0x5555)
    t.insert(dev(keys), dev(vals))
    t.erase(dev(keys[::5]))
    return t, keys, vals


def test_save_load_round_trip(tmp_path):
    rng = np.random.default_rng(1)
    t, keys, vals = filled_map(rng)
    path = tmp_path / "map.sgt"
    t.save(path)
    g = t.geometry()
    # header, device header, slot image, then the excess-list accounting's bit arrays (on at this size)
    assert t.excess_used() >= 0
    acct = (g.bucket_count + 31) // 32 * 4 + (g.num_groups * g.slots_per_group + 2 + 31) // 32 * 4
    assert path.stat().st_size == 128 + 64 + (g.num_groups + 1) * 128 + acct
    u = sg.unordered_map.load(path)
    assert u.kind == t.kind and u.size() == t.size() and u.valid() and u.excess_used() == t.excess_used()
    assert u.max_size() == t.max_size() and u.bucket_count() == t.bucket_count()
    # same slots, in the same order
    assert torch.equal(u.device_range(), t.device_range())
    q = np.concatenate([keys, rng.integers(0, 2**64 - 1, size=5000, dtype=np.uint64)])
    tv, tf = t.find(dev(q))
    uv, uf = u.find(dev(q))
    assert torch.equal(tf, uf) and torch.equal(tv[tf.bool()], uv[uf.bool()])
    assert t.status()[2] == u.status()[2]  # erased slots awaiting reuse
    # the loaded table is live: after the same inserts both hold the same elements (which slot a key
    # takes when keys race for one group is not fixed)
    more = rng.integers(0, 2**64 - 1, size=3000, dtype=np.uint64)
    for x in (t, u):
        x.insert(dev(more), dev(more))
    assert t.size() == u.size() and u.valid()
    tk, tv2 = t.range_copy()
    uk, uv2 = u.range_copy()
    to, uo = torch.argsort(tk), torch.argsort(uk)
    assert torch.equal(tk[to], uk[uo]) and torch.equal(tv2[to], uv2[uo])
    for x in (t, u):
        sg.unordered_base.destroyDeviceObject(x)


def test_custom_hash_table_round_trip(tmp_path):
    rng = np.random.default_rng(2)
    k = np.zeros(5000, O.VEC3I16)
    c = rng.integers(-30, 30, size=(5000, 3)).astype(np.int16)
    k["x"], k["y"], k["z"] = c[:, 0], c[:, 1], c[:, 2]
    w, h = O.vec3i16_words(k), O.spatial_hash(k)
    t = sg.unordered_set.createDeviceObject(1 << 14, key="u64", custom_hash=True)
    t.insert(dev(w), hashes=dev(h))
    t.save(tmp_path / "set.sgt")
    u = sg.unordered_set.load(tmp_path / "set.sgt")
    assert u.custom_hash and u.size() == t.size()
    assert bool(u.contains(dev(w), hashes=dev(h)).bool().all())
    for x in (t, u):
        sg.unordered_base.destroyDeviceObject(x)


@pytest.mark.parametrize("new_cap", [1 << 18, 50000])
def test_rehash_keeps_every_element(new_cap):
    rng = np.random.default_rng(3)
    t, keys, vals = filled_map(rng)
    before_keys, before_vals = t.range_copy()
    n = t.size()
    t.rehash(new_cap)
    assert t.size() == n and t.valid()
    assert t.geometry().capacity == new_cap
    assert t.bucket_count() == sg.geometry_for(N.MAP_U64_U64, new_cap).bucket_count
    v, f = t.find(before_keys)
    assert bool(f.bool().all()) and torch.equal(v, before_vals)
    sg.unordered_base.destroyDeviceObject(t)


def test_rehash_too_small_refuses_and_keeps_the_table():
    rng = np.random.default_rng(4)
    t, keys, vals = filled_map(rng)
    n = t.size()
    rng_before = t.device_range().clone()
    with pytest.raises(N.StdgpuError) as e:
        t.rehash(1000)
    assert e.value.status == N.SG_ERR_FULL
    assert t.size() == n and torch.equal(t.device_range(), rng_before) and t.valid()
    sg.unordered_base.destroyDeviceObject(t)

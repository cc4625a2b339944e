"""Custom key types with a user hash on the GPU: 3 x int16 keys stored as 8-byte key words, buckets from the
spatial hash passed per key (sg_unordered_*_hashed), against the oracle fed the same words and hashes (the
oracle is pinned against the reference's unordered_set / unordered_map<Key, T, Hash> in test_oracle.py)."""

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

from gpu_util import dev, host, per_key_success

pytestmark = pytest.mark.gpu


def vec_keys(rng, n, lo=-40, hi=40):
    c = rng.integers(lo, hi, size=(n, 3)).astype(np.int16)
    k = np.zeros(n, O.VEC3I16)
    k["x"], k["y"], k["z"] = c[:, 0], c[:, 1], c[:, 2]
    return k


@pytest.mark.parametrize("kind", [O.SET_VEC3I16, O.MAP_VEC3I16_U32])
def test_hashed_matches_oracle(kind):
    rng = np.random.default_rng(kind)
    cap = 1 << 17
    wk = O.WORD_KIND[kind]
    is_map = O.VAL_DTYPE[kind] is not None
    t = (sg.unordered_map.createDeviceObject(cap, key="u64", mapped="u32", custom_hash=True) if is_map
         else sg.unordered_set.createDeviceObject(cap, key="u64", custom_hash=True))
    port = O.PortTable(wk, cap)
    for rnd in range(3):
        k = vec_keys(rng, 30000)
        w, h = O.vec3i16_words(k), O.spatial_hash(k)
        v = (w & np.uint64(0xFFFFFFFF)).astype(np.uint32) if is_map else None
        f = torch.zeros(len(w), dtype=torch.uint8, device="cuda")
        t.insert(dev(w), dev(v) if is_map else None, flags=f, hashes=dev(h))
        pf = port.insert(w, v, flags=True, hashes=h)
        assert per_key_success(w, f.cpu().numpy()) == per_key_success(w, pf)
        e = vec_keys(rng, 8000)
        we, he = O.vec3i16_words(e), O.spatial_hash(e)
        fe = torch.zeros(len(we), dtype=torch.uint8, device="cuda")
        t.erase(dev(we), flags=fe, hashes=dev(he))
        pe = port.erase(we, flags=True, hashes=he)
        assert per_key_success(we, fe.cpu().numpy()) == per_key_success(we, pe)
        assert t.size() == port.size()
    q = vec_keys(rng, 20000, -45, 45)
    wq, hq = O.vec3i16_words(q), O.spatial_hash(q)
    gv, gf = t.find(dev(wq), hashes=dev(hq))
    pv, pf = port.find(wq, hashes=hq)
    assert np.array_equal(gf.cpu().numpy(), pf)
    if is_map:
        assert np.array_equal(host(gv, np.uint32)[pf == 1], pv[pf == 1])
    assert np.array_equal(t.contains(dev(wq), hashes=dev(hq)).cpu().numpy(), pf)
    assert t.valid()
    rk, _ = t.range_copy()
    pk, _ = port.range()
    assert np.array_equal(np.sort(host(rk, np.uint64)), np.sort(pk))
    # bucket() of a custom key is the fibonacci hashing of its hash
    assert t.bucket_of_hash(int(hq[0])) == port.bucket(int(hq[0]))
    sg.unordered_base.destroyDeviceObject(t)


def test_hashed_table_rejects_identity_calls():
    t = sg.unordered_set.createDeviceObject(1024, key="u64", custom_hash=True)
    lib = sg.load()
    keys = dev(np.arange(10, dtype=np.uint64))
    from ctypes import c_void_p
    assert lib.sg_unordered_insert_kv(t._h, c_void_p(keys.data_ptr()), None, 10, None, None) == N.SG_ERR_BAD_ARG
    assert lib.sg_unordered_contains(t._h, c_void_p(keys.data_ptr()), 10, None, None) == N.SG_ERR_BAD_ARG
    with pytest.raises(ValueError):
        t.insert(keys)  # no hashes
    sg.unordered_base.destroyDeviceObject(t)
    u = sg.unordered_set.createDeviceObject(1024, key="u64")
    hs = dev(np.arange(10, dtype=np.uint64))
    assert lib.sg_unordered_insert_hashed(u._h, c_void_p(keys.data_ptr()), None, c_void_p(hs.data_ptr()), 10, None,
                                          None) == N.SG_ERR_BAD_ARG
    sg.unordered_base.destroyDeviceObject(u)

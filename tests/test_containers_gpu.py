"""vector push_back, deque push_back / pop_front and bitset count on the GPU against the oracle."""

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg

from gpu_util import dev

pytestmark = pytest.mark.gpu


def test_vector_push_back_matches_reference(golden):
    """push_back_some/all/too_many (tests/stdgpu/vector.inc:404-512): size, which elements fit, contents."""
    g = golden("vector.npz")
    values, pred = g["values"], g["pred"]
    for cap in [100, 1000, 5000]:
        v = sg.vector.createDeviceObject(cap, elem_bytes=4)
        flags = torch.zeros(len(values), dtype=torch.uint8, device="cuda")
        v.push_back(dev(values), dev(pred), flags=flags)
        assert v.size() == int(g[f"size_{cap}"])
        f = flags.cpu().numpy()
        assert f.sum() == g[f"pushed_{cap}"].sum()
        assert np.all(f <= pred)
        got = np.sort(v.data().cpu().numpy().view(np.uint32))
        # the pushed elements, whichever fitted, are exactly the stored contents
        assert np.array_equal(got, np.sort(values[f == 1]))
        if cap == 5000:
            assert np.array_equal(got, np.sort(g[f"contents_{cap}"]))
        sg.vector.destroyDeviceObject(v)


def test_vector_push_back_predicate_large():
    n = 1 << 24
    rng = np.random.default_rng(3)
    pred = (rng.random(n) < 0.3).astype(np.uint8)
    values = np.arange(n, dtype=np.uint32)
    v = sg.vector.createDeviceObject(n, elem_bytes=4)
    v.push_back(dev(values), dev(pred))
    assert v.size() == int(pred.sum())
    got = np.sort(v.data().cpu().numpy().view(np.uint32))
    assert np.array_equal(got, np.nonzero(pred)[0].astype(np.uint32))
    sg.vector.destroyDeviceObject(v)


def test_deque_matches_reference_sequential_semantics(golden):
    """Initial fill then a mixed launch: the multiset of (popped + remaining) equals (initial + pushed),
    and counts match the reference, which ran the same ops one at a time."""
    g = golden("deque.npz")
    cap = int(g["capacity"])
    d = sg.deque.createDeviceObject(cap, elem_bytes=8)
    init = g["init"]
    d.ops(None, dev(init))
    assert d.size() == len(init)
    # one parallel launch: element order follows ticket order, not index order
    assert np.array_equal(np.sort(d.to_tensor().cpu().numpy().view(np.uint64)), np.sort(init))
    popped, ok = d.ops(dev(g["is_push"]), dev(g["values"]))
    ok = ok.cpu().numpy()
    popped = popped.cpu().numpy().view(np.uint64)
    is_push = g["is_push"].astype(bool)
    remaining = d.to_tensor().cpu().numpy().view(np.uint64)
    assert d.size() == len(remaining)
    pushed_vals = g["values"][is_push & (ok == 1)]
    popped_vals = popped[~is_push & (ok == 1)]
    lhs = np.sort(np.concatenate([popped_vals, remaining]))
    rhs = np.sort(np.concatenate([init, pushed_vals]))
    assert np.array_equal(lhs, rhs)
    # counts are consistent; when every op succeeded (as in the reference's one-at-a-time run),
    # the final size is the reference's
    assert d.size() == len(init) + int((is_push & (ok == 1)).sum()) - int((~is_push & (ok == 1)).sum())
    if ok.sum() == g["ok"].sum() == len(ok):
        assert d.size() == int(g["size"])
    sg.deque.destroyDeviceObject(d)


def test_deque_fifo_order_across_launches():
    """FIFO holds between launches: everything pushed by an earlier launch leaves before a later launch's."""
    d = sg.deque.createDeviceObject(1000, elem_bytes=8)
    a = np.arange(1, 701, dtype=np.uint64)
    d.ops(None, dev(a))
    popped, ok = d.ops(dev(np.zeros(300, np.uint8)), dev(np.zeros(300, np.uint64)))
    assert ok.cpu().numpy().sum() == 300
    p = popped.cpu().numpy().view(np.uint64)
    assert len(np.unique(p)) == 300 and np.isin(p, a).all()
    b = np.arange(1000, 1500, dtype=np.uint64)
    d.ops(None, dev(b))  # wraps around the ring
    rem = d.to_tensor().cpu().numpy().view(np.uint64)
    assert len(rem) == 900
    assert np.array_equal(np.sort(rem[:400]), np.setdiff1d(a, p))
    assert np.array_equal(np.sort(rem[400:]), b)
    # over-full: 1000 - 900 = 100 fit
    _, ok = d.ops(None, dev(np.arange(200, dtype=np.uint64)))
    assert ok.cpu().numpy().sum() == 100 and d.size() == 1000
    # over-empty pops report failure
    _, ok = d.ops(dev(np.zeros(1200, np.uint8)), dev(np.zeros(1200, np.uint64)))
    assert ok.cpu().numpy().sum() == 1000 and d.size() == 0
    sg.deque.destroyDeviceObject(d)


def test_deque_mixed_large_conservation():
    n = 1 << 22
    rng = np.random.default_rng(9)
    cap = 1 << 21
    d = sg.deque.createDeviceObject(cap, elem_bytes=8)
    init = rng.integers(0, 2**62, size=cap // 2, dtype=np.uint64)
    d.ops(None, dev(init))
    is_push = (rng.random(n) < 0.5).astype(np.uint8)
    values = rng.integers(0, 2**62, size=n, dtype=np.uint64)
    popped, ok = d.ops(dev(is_push), dev(values))
    ok = ok.cpu().numpy().astype(bool)
    popped = popped.cpu().numpy().view(np.uint64)
    rem = d.to_tensor().cpu().numpy().view(np.uint64)
    ip = is_push.astype(bool)
    lhs = np.sort(np.concatenate([popped[~ip & ok], rem]))
    rhs = np.sort(np.concatenate([init, values[ip & ok]]))
    assert np.array_equal(lhs, rhs)
    assert d.size() == len(init) + (ip & ok).sum() - (~ip & ok).sum()
    sg.deque.destroyDeviceObject(d)


def test_bitset_count_matches_reference(golden):
    g = golden("bitset.npz")
    for nbits in [1, 31, 32, 33, 1000, 4096, 100003]:
        assert sg.bitset_count(dev(g[f"words_{nbits}"]), nbits) == int(g[f"count_{nbits}"])


@pytest.mark.parametrize("nbits", [0, 1, 127, 128, 129, (1 << 20) + 5, (1 << 30) + 17])
def test_bitset_count_against_oracle(nbits):
    rng = np.random.default_rng(nbits % 1000)
    words = rng.integers(0, 2**32, size=max((nbits + 31) // 32, 1), dtype=np.uint64).astype(np.uint32)
    assert sg.bitset_count(dev(words), nbits) == O.port_bitset_count(words, nbits)


def test_bitset_count_2_pow_33_bits():
    """2^33 bits (1 GiB of blocks): the count exceeds the reference's 32-bit index_t, here int64."""
    nblocks = 1 << 28
    g = torch.Generator(device="cuda").manual_seed(5)
    words = torch.randint(-(2**31), 2**31, (nblocks,), dtype=torch.int32, device="cuda", generator=g)
    got = sg.bitset_count(words, nblocks * 32)
    # popcount by torch integer ops as an independent check
    x = words.view(torch.int32).to(torch.int64) & 0xFFFFFFFF
    cnt = torch.zeros_like(x)
    for b in range(32):
        cnt += (x >> b) & 1
    assert got == int(cnt.sum())

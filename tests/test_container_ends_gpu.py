"""deque push_front / pop_back beside push_back / pop_front, vector pop_back / insert / erase, and the
queue / stack adapters, against the oracle (pinned to the reference's deque in test_oracle.py)."""

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

from gpu_util import dev, host

pytestmark = pytest.mark.gpu


def runs(ops):
    """(op, start, stop) of maximal runs of one operation."""
    out, i = [], 0
    while i < len(ops):
        j = i
        while j < len(ops) and ops[j] == ops[i]:
            j += 1
        out.append((int(ops[i]), i, j))
        i = j
    return out


def test_deque_batches_replay_the_reference_sequence(golden):
    """Each batch holds one operation and at most one 2048-element tile, so a launch acts exactly like the
    calls of its batch made in order; the replay must give the reference's answers element by element."""
    g = golden("deque_ends.npz")
    cap = int(g["capacity"])
    d = sg.deque.createDeviceObject(cap, elem_bytes=8)
    d.push_back(dev(g["init"]))
    ops, values = g["ops"], g["values"]
    popped = np.zeros(len(ops), np.uint64)
    ok = np.zeros(len(ops), np.uint8)
    for op, a, b in runs(ops):
        n = b - a
        if op == 1:
            ok[a:b] = d.push_back(dev(values[a:b])).cpu().numpy()
        elif op == 2:
            ok[a:b] = d.push_front(dev(values[a:b])).cpu().numpy()
        else:
            v, f = d.pop_front(n) if op == 0 else d.pop_back(n)
            ok[a:b] = f.cpu().numpy()
            popped[a:b] = np.where(ok[a:b] == 1, host(v, np.uint64), 0)
    assert np.array_equal(ok, g["ok"])
    assert np.array_equal(popped, g["popped"])
    assert d.size() == int(g["size"])
    assert np.array_equal(host(d.to_tensor(), np.uint64), g["remaining"])
    sg.deque.destroyDeviceObject(d)


def test_deque_large_end_batches_against_oracle():
    """push_front / pop_back launches of many tiles stay exact (element i is the i-th call); FIFO launches
    between them are checked as multisets."""
    rng = np.random.default_rng(11)
    cap = 1 << 18
    d = sg.deque.createDeviceObject(cap, elem_bytes=4)
    model = []
    for rnd in range(6):
        v = rng.integers(0, 2**32, size=int(rng.integers(1, 100000)), dtype=np.uint64).astype(np.uint32)
        ok = d.push_front(dev(v)).cpu().numpy()
        k = int(ok.sum())
        assert np.all(ok[:k] == 1) and np.all(ok[k:] == 0)
        model = list(v[:k][::-1]) + model
        m = int(rng.integers(1, 120000))
        pv, pf = d.pop_back(m)
        kk = int(pf.cpu().numpy().sum())
        assert kk == min(m, len(model))
        want = model[len(model) - kk:][::-1]
        assert np.array_equal(host(pv, np.uint32)[:kk], np.array(want, np.uint32))
        model = model[: len(model) - kk]
        assert d.size() == len(model)
        assert np.array_equal(host(d.to_tensor(), np.uint32), np.array(model, np.uint32))
    sg.deque.destroyDeviceObject(d)


def test_vector_pop_back_insert_erase():
    v = sg.vector.createDeviceObject(5000, elem_bytes=4)
    first = np.arange(1000, dtype=np.uint32) * 3
    v.push_back(dev(first))
    vals, ok = v.pop_back(300)
    assert ok.cpu().numpy().all()
    assert np.array_equal(host(vals, np.uint32), first[::-1][:300])
    assert v.size() == 700
    more = np.arange(10, dtype=np.uint32) + 100000
    v.insert(dev(more))
    assert v.size() == 710
    assert np.array_equal(host(v.data(), np.uint32), np.concatenate([first[:700], more]))
    with pytest.raises(N.StdgpuError) as e:
        v.insert(dev(np.zeros(5000, np.uint32)))
    assert e.value.status == N.SG_ERR_FULL and v.size() == 710
    v.erase(10)
    assert v.size() == 700
    with pytest.raises(N.StdgpuError):
        v.erase(701)
    vals, ok = v.pop_back(1000)
    assert int(ok.sum()) == 700 and v.size() == 0
    assert np.array_equal(host(vals, np.uint32)[:700], first[:700][::-1])
    sg.vector.destroyDeviceObject(v)


def test_queue_and_stack_adapters():
    q = sg.queue.createDeviceObject(100, elem_bytes=8)
    s = sg.stack.createDeviceObject(100, elem_bytes=8)
    x = np.arange(1, 41, dtype=np.uint64)
    assert q.push(dev(x)).cpu().numpy().all() and s.push(dev(x)).cpu().numpy().all()
    qv, qf = q.pop(10)
    sv, sf = s.pop(10)
    assert np.array_equal(host(qv, np.uint64), x[:10])          # first in, first out
    assert np.array_equal(host(sv, np.uint64), x[::-1][:10])    # last in, first out
    assert q.size() == 30 and s.size() == 30 and not q.empty()
    sg.queue.destroyDeviceObject(q)
    sg.stack.destroyDeviceObject(s)


def test_mixed_launches_on_small_deques_keep_the_multiset():
    """Mixed push_back / pop_front launches of thousands of operations on deques of 64-1000 elements: the
    ring wraps inside one tile and runs near empty, so one thread may hold a pop and the push of the same
    ticket, or a push and the pop one lap earlier.  Every launch keeps the multiset (popped + remaining ==
    before + pushed), stays within capacity, and leaves no wait error (size() would report it)."""
    gen = torch.Generator(device="cuda").manual_seed(3)
    for cap in (64, 100, 1000):
        d = sg.deque.createDeviceObject(cap, elem_bytes=8)
        for it in range(30):
            n = int(torch.randint(512, 8192, (1,), generator=gen, device="cuda").item())
            frac = [0.5, 0.6, 0.4][it % 3]
            is_push = (torch.rand(n, device="cuda", generator=gen) < frac).to(torch.uint8)
            vals = torch.randint(0, 1 << 62, (n,), dtype=torch.int64, device="cuda", generator=gen)
            before = d.to_tensor()
            popped, ok = d.ops(is_push, vals)
            size = d.size()
            after = d.to_tensor()
            ip, okb = is_push.bool(), ok.bool()
            lhs = torch.sort(torch.cat([popped[~ip & okb], after])).values
            rhs = torch.sort(torch.cat([before, vals[ip & okb]])).values
            assert torch.equal(lhs, rhs), (cap, it)
            assert size == len(after) <= cap
        sg.deque.destroyDeviceObject(d)

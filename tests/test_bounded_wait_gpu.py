"""Failure detection without a GPU fault: a deque slot whose turn word never arrives.

The turn word of the slot the next pop_front will use is overwritten from the host with a value no push
will ever store (a flag that nothing sets).  The pop's bounded wait runs out (about a second), the launch
returns normally, the pop reports failure, the deque's error bit makes size() return
SG_ERR_RETRY_EXHAUSTED, and the context stays usable: other containers keep working."""

import ctypes

import numpy as np
import pytest
import torch

import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

from gpu_util import dev, host

pytestmark = pytest.mark.gpu


def test_wait_that_runs_out_reports_and_leaves_the_context_usable():
    d = sg.deque.createDeviceObject(64, elem_bytes=8)
    d.push_back(dev(np.arange(1, 11, dtype=np.uint64)))
    assert d.size() == 10
    v = N.sg_deque_view()
    N.check(sg.load().sg_deque_view_of(d._h, ctypes.byref(v)), "view")
    # device memory seen as tensors: counters (int64 size, uint64 begin, ...) and the turn words
    from stdgpu_gb300.containers import _DeviceArray
    counters = torch.as_tensor(_DeviceArray(v.counters, 2, 8), device="cuda")
    seq = torch.as_tensor(_DeviceArray(v.seq, 64, 4), device="cuda")
    torch.cuda.synchronize()
    begin = int(counters[1].item()) & (2**64 - 1)  # the next pop_front takes ticket `begin`
    seq[begin % 64] = 0x7FFFFFFF  # a turn value no push stores for this slot
    torch.cuda.synchronize()
    popped, ok = d.pop_front(1)
    torch.cuda.synchronize()
    assert int(ok[0]) == 0
    with pytest.raises(N.StdgpuError) as e:
        d.size()
    assert e.value.status == N.SG_ERR_RETRY_EXHAUSTED
    sg.deque.destroyDeviceObject(d)
    # the context is still usable
    t = sg.unordered_set.createDeviceObject(1 << 12, key="u64")
    t.insert(dev(np.arange(100, dtype=np.uint64)))
    assert t.size() == 100 and t.valid()
    sg.unordered_base.destroyDeviceObject(t)

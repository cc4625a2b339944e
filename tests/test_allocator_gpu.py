"""Container storage through PyTorch's caching allocator: tables, vectors and deques take their device
memory from torch, hand it back on destroy, and the pair cannot be swapped while any of it is allocated.
Runs in a fresh process: the allocator can only change while the library holds no storage."""

import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

SCENARIO = r'''
import sys
sys.path.insert(0, sys.argv[1])
sys.path.insert(0, sys.argv[1] + "/tests")
import numpy as np, torch
import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N
from gpu_util import dev
torch.cuda.synchronize()
base = torch.cuda.memory_allocated()
assert sg.live_device_allocations() == 0
sg.use_torch_allocator(True)
t = sg.unordered_map.createDeviceObject(1 << 20, key="u64", mapped="u32")
v = sg.vector.createDeviceObject(1 << 16, elem_bytes=4)
d = sg.deque.createDeviceObject(1 << 16, elem_bytes=8)
assert sg.live_device_allocations() > 0
assert torch.cuda.memory_allocated() - base >= t.geometry().storage_bytes
try:
    sg.use_torch_allocator(False)
    raise SystemExit("allocator swapped while storage was allocated")
except N.StdgpuError as e:
    assert e.status == N.SG_ERR_BAD_ARG
keys = np.arange(1, 300001, dtype=np.uint64)
t.insert(dev(keys), dev((keys & 0xFFFF).astype(np.uint32)))
vals, found = t.find(dev(keys))
assert bool(found.bool().all()) and t.valid()
v.push_back(dev(np.arange(1000, dtype=np.uint32)))
assert v.size() == 1000
d.push_back(dev(np.arange(10, dtype=np.uint64)))
assert d.size() == 10
del vals, found
torch.cuda.synchronize()
held = torch.cuda.memory_allocated() - base
sg.unordered_base.destroyDeviceObject(t)
sg.vector.destroyDeviceObject(v)
sg.deque.destroyDeviceObject(d)
assert sg.live_device_allocations() == 0
torch.cuda.synchronize()
# everything the containers held went back to torch
assert torch.cuda.memory_allocated() == base, (held, torch.cuda.memory_allocated() - base)
sg.use_torch_allocator(False)
print("OK")
'''


def test_containers_allocate_through_torch():
    r = subprocess.run([sys.executable, "-c", SCENARIO, str(ROOT)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "OK" in r.stdout, r.stdout + r.stderr

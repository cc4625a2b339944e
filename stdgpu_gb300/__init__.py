"""stdgpu_gb300: GB300-native (sm_103a) hashed containers with the reference stdgpu API.

The compute path is the native library built from ``stdgpu_gb300/csrc`` and
reached through its C ABI (``include/stdgpu_gb300.h``); this package holds the
Python mirror of the reference's host API over that ABI.
"""

from .containers import (  # noqa: F401
    KINDS,
    bitset_count,
    default_stager,
    deque,
    geometry_for,
    kernel_launch_count,
    live_device_allocations,
    queue,
    stack,
    stager,
    table_batch,
    unordered_base,
    unordered_map,
    unordered_set,
    use_torch_allocator,
    vector,
)
from ._native import StdgpuError, library_path, load  # noqa: F401

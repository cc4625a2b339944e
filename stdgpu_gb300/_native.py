"""ctypes binding of the C ABI in ``include/stdgpu_gb300.h``.

The shared library is built in-tree (``stdgpu_gb300/_lib``).  There is no
fallback: if the library cannot be loaded, every entry point raises.
"""

from __future__ import annotations

import ctypes
from ctypes import c_uint64, POINTER, c_char_p, c_int32, c_int64, c_uint8, c_uint32, c_void_p
from pathlib import Path

from . import build as _build

SG_OK = 0
SG_ERR_FULL = 1
SG_ERR_BAD_ARG = 2
SG_ERR_OOM = 3
SG_ERR_BUDGET = 4
SG_ERR_RETRY_EXHAUSTED = 5
SG_ERR_CUDA = 6
SG_ERR_NO_DEVICE = 7

SET_U32, SET_U64, MAP_U64_U32, MAP_U64_U64, MAP_U32_U32, MAP_U32_U64 = range(6)


class sg_allocator(ctypes.Structure):
    _fields_ = [("alloc", c_void_p), ("release", c_void_p), ("ctx", c_void_p), ("release_ctx", c_void_p)]


class sg_geometry(ctypes.Structure):
    _fields_ = [
        ("capacity", c_int64),
        ("bucket_count", c_int64),
        ("excess_count", c_int64),
        ("max_size", c_int64),
        ("num_groups", c_int64),
        ("slot_bytes", c_int32),
        ("slots_per_group", c_int32),
        ("storage_bytes", c_int64),
    ]


class sg_unordered_view(ctypes.Structure):
    _fields_ = [
        ("slots", c_void_p),
        ("header", c_void_p),
        ("num_groups", c_int64),
        ("total_count", c_int64),
        ("bucket_count", c_int64),
        ("bucket_bits", c_int32),
        ("kind", c_int32),
        ("insert_locks", c_void_p),
        ("lock_mask", c_int64),
        ("bucket_heads", c_void_p),
        ("slot_heads", c_void_p),
        ("excess_count", c_int64),
    ]


class sg_vector_view(ctypes.Structure):
    _fields_ = [("data", c_void_p), ("size", c_void_p), ("capacity", c_int64), ("elem_bytes", c_int32),
                ("pad", c_int32), ("slot_state", c_void_p), ("sync", c_void_p)]


class sg_deque_view(ctypes.Structure):
    _fields_ = [("data", c_void_p), ("seq", c_void_p), ("counters", c_void_p), ("capacity", c_int64),
                ("elem_bytes", c_int32), ("pad", c_int32), ("slot_state", c_void_p), ("sync", c_void_p)]


class sg_request(ctypes.Structure):
    _fields_ = [("table", c_int32), ("op", c_int32), ("n", c_int64), ("keys", c_void_p), ("mapped", c_void_p),
                ("out_mapped", c_void_p), ("out_flags", c_void_p)]


class sg_server_stats(ctypes.Structure):
    _fields_ = [("requests_done", c_int64), ("keys_done", c_int64), ("p50_us", ctypes.c_double),
                ("p99_us", ctypes.c_double), ("max_us", ctypes.c_double), ("keys_per_s", ctypes.c_double),
                ("launches", c_int64), ("waves", c_int64), ("refused_budget", c_int64), ("rehashes", c_int64),
                ("hbm_used_bytes", c_int64), ("grow_host_us", ctypes.c_double),
                ("max_grow_host_us", ctypes.c_double), ("grow_create_us", ctypes.c_double)]


# name -> (restype, argtypes); every symbol the header declares
SIGNATURES = {
    "sg_set_device_allocator": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "sg_live_device_allocations": (c_int64, []),
    "sg_unordered_create": (c_int32, [c_int32, c_int64, c_void_p, POINTER(c_void_p)]),
    "sg_unordered_create_with_allocator": (c_int32, [c_int32, c_int64, c_int32, POINTER(sg_allocator), c_void_p,
                                                   POINTER(c_void_p)]),
    "sg_unordered_destroy": (c_int32, [c_void_p]),
    "sg_unordered_insert": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_insert_kv": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_erase": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_set_insert_mode": (c_int32, [c_void_p, c_int32]),
    "sg_unordered_create_hashed": (c_int32, [c_int32, c_int64, c_void_p, POINTER(c_void_p)]),
    "sg_unordered_insert_hashed": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_erase_hashed": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_find_hashed": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "sg_unordered_contains_hashed": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_bucket_of_hash": (c_int32, [c_void_p, c_uint64, POINTER(c_int64)]),
    "sg_unordered_is_hashed": (c_int32, [c_void_p, POINTER(c_int32)]),
    "sg_unordered_rehash": (c_int32, [c_void_p, c_int64, c_void_p]),
    "sg_unordered_save": (c_int32, [c_void_p, c_char_p, c_void_p]),
    "sg_unordered_load": (c_int32, [c_char_p, c_void_p, POINTER(c_void_p)]),
    "sg_unordered_find": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "sg_unordered_contains": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_size": (c_int32, [c_void_p, c_void_p, POINTER(c_int64)]),
    "sg_unordered_status": (c_int32, [c_void_p, c_void_p, POINTER(c_int64), POINTER(c_int64)]),
    "sg_unordered_clear": (c_int32, [c_void_p, c_void_p]),
    "sg_unordered_valid": (c_int32, [c_void_p, c_void_p, POINTER(c_int32)]),
    "sg_unordered_device_range": (c_int32, [c_void_p, c_void_p, c_void_p, POINTER(c_int64)]),
    "sg_unordered_range_copy": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, POINTER(c_int64)]),
    "sg_unordered_bucket": (c_int32, [c_void_p, c_void_p, POINTER(c_int64)]),
    "sg_unordered_geometry": (c_int32, [c_void_p, POINTER(sg_geometry)]),
    "sg_unordered_view_of": (c_int32, [c_void_p, POINTER(sg_unordered_view)]),
    "sg_unordered_set_excess_accounting": (c_int32, [c_void_p, c_int32, c_void_p]),
    "sg_unordered_excess_used": (c_int32, [c_void_p, c_void_p, POINTER(c_int64)]),
    "sg_unordered_call_scratch": (c_int32, [c_void_p, c_int64, c_void_p, POINTER(c_void_p)]),
    "sg_unordered_geometry_for": (c_int32, [c_int32, c_int64, POINTER(sg_geometry)]),
    "sg_stager_create": (c_int32, [c_int64, c_int32, POINTER(c_void_p)]),
    "sg_stager_destroy": (c_int32, [c_void_p]),
    "sg_stager_set_inputs_ready": (c_int32, [c_void_p, c_int32]),
    "sg_unordered_insert_host": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_insert_kv_host": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_erase_host": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_unordered_find_host": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "sg_unordered_contains_host": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_batch_create": (c_int32, [c_int32, c_int32, c_void_p, c_void_p, POINTER(c_void_p)]),
    "sg_batch_destroy": (c_int32, [c_void_p]),
    "sg_batch_configure": (c_int32, [c_void_p, c_int32, c_int32, c_int32]),
    "sg_batch_clear": (c_int32, [c_void_p, c_void_p]),
    "sg_batch_insert": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sg_batch_insert_kv": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sg_batch_erase": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sg_batch_find": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sg_batch_contains": (c_int32, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "sg_batch_sizes": (c_int32, [c_void_p, c_void_p, c_void_p]),
    "sg_batch_view_of": (c_int32, [c_void_p, c_int32, POINTER(sg_unordered_view)]),
    "sg_batch_info": (c_int32, [c_void_p, POINTER(c_int64), POINTER(c_int32)]),
    "sg_server_create": (c_int32, [c_int32, c_int64, c_int32, c_int32, POINTER(c_void_p)]),
    "sg_server_destroy": (c_int32, [c_void_p]),
    "sg_server_admit_table": (c_int32, [c_void_p, c_int32, c_int64]),
    "sg_server_drop_table": (c_int32, [c_void_p, c_int32]),
    "sg_server_submit": (c_int32, [c_void_p, POINTER(sg_request), POINTER(c_int64)]),
    "sg_server_submit_many": (c_int32, [c_void_p, POINTER(sg_request), c_int32, POINTER(c_int64)]),
    "sg_server_set_paused": (c_int32, [c_void_p, c_int32]),
    "sg_server_set_policy": (c_int32, [c_void_p, c_int64, c_int64, c_int32, c_int32]),
    "sg_server_set_grow_ahead": (c_int32, [c_void_p, c_int32]),
    "sg_server_wait": (c_int32, [c_void_p, c_int64, c_int32, POINTER(c_int32)]),
    "sg_server_drain": (c_int32, [c_void_p, c_int32]),
    "sg_server_get_stats": (c_int32, [c_void_p, POINTER(sg_server_stats)]),
    "sg_server_request_latency": (c_int32, [c_void_p, c_int64, POINTER(ctypes.c_double)]),
    "sg_server_table_size": (c_int32, [c_void_p, c_int32, POINTER(c_int64)]),
    "sg_server_table_view": (c_int32, [c_void_p, c_int32, POINTER(sg_unordered_view)]),
    "sg_vector_create": (c_int32, [c_int32, c_int64, POINTER(c_void_p)]),
    "sg_vector_create_with_allocator": (c_int32, [c_int32, c_int64, POINTER(sg_allocator), POINTER(c_void_p)]),
    "sg_vector_pop_back": (c_int32, [c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "sg_vector_insert": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p]),
    "sg_vector_erase": (c_int32, [c_void_p, c_int64, c_void_p]),
    "sg_deque_push_front": (c_int32, [c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_deque_pop_back": (c_int32, [c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "sg_vector_destroy": (c_int32, [c_void_p]),
    "sg_vector_push_back": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_vector_size": (c_int32, [c_void_p, c_void_p, POINTER(c_int64)]),
    "sg_vector_clear": (c_int32, [c_void_p, c_void_p]),
    "sg_vector_view_of": (c_int32, [c_void_p, POINTER(sg_vector_view)]),
    "sg_deque_create": (c_int32, [c_int32, c_int64, POINTER(c_void_p)]),
    "sg_deque_create_with_allocator": (c_int32, [c_int32, c_int64, POINTER(sg_allocator), POINTER(c_void_p)]),
    "sg_deque_destroy": (c_int32, [c_void_p]),
    "sg_deque_ops": (c_int32, [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p, c_void_p]),
    "sg_deque_size": (c_int32, [c_void_p, c_void_p, POINTER(c_int64)]),
    "sg_deque_copy_out": (c_int32, [c_void_p, c_void_p, c_void_p, POINTER(c_int64)]),
    "sg_deque_clear": (c_int32, [c_void_p, c_void_p]),
    "sg_deque_view_of": (c_int32, [c_void_p, POINTER(sg_deque_view)]),
    "sg_bitset_count": (c_int32, [c_void_p, c_int64, c_void_p, POINTER(c_int64)]),
    "sg_bitset_count_noalloc": (c_int32, [c_void_p, c_int64, c_void_p, c_void_p]),
    "sg_measure_random_reads": (c_int32, [c_int64, c_int64, c_int32, c_void_p, c_void_p]),
    "sg_kernel_launch_count": (c_int64, []),
    "sg_status_string": (c_char_p, [c_int32]),
}

_lib: ctypes.CDLL | None = None


class StdgpuError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = _lib.sg_status_string(status).decode() if _lib is not None else str(status)
        super().__init__(f"{where}: {msg} (status {status})")


def library_path() -> Path:
    """The in-tree library, or the file named by $STDGPU_GB300_LIB (a separately built copy)."""
    import os
    override = os.environ.get("STDGPU_GB300_LIB")
    return Path(override) if override else _build.library_path()


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load (building first when needed) the product library; raises when it is unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    path = library_path()
    import os
    if os.environ.get("STDGPU_GB300_LIB"):
        build_if_missing = False
    elif not path.exists() or (build_if_missing and not _build.is_current()):
        if not build_if_missing:
            raise RuntimeError(f"stdgpu_gb300 native library missing: {path}")
        _build.build()
    lib = ctypes.CDLL(str(path))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int, where: str, allow: tuple[int, ...] = ()) -> int:
    if status != SG_OK and status not in allow:
        raise StdgpuError(status, where)
    return status

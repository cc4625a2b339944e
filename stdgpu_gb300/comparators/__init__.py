"""The plain one-call-per-table paths driven from native code (plain_calls.cpp), the comparators of the
batched and served modes: the same C-ABI calls a C++ caller makes, in a C++ loop."""

from __future__ import annotations

import ctypes
from ctypes import POINTER, c_double, c_float, c_int32, c_int64, c_void_p

import numpy as np

from .. import _native as N
from .. import build as _build

_lib = None


def load() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        N.load()  # the product library first (the comparators link against it)
        path = _build.OUT / _build.COMPARATORS_LIB
        if not path.exists():
            _build.build_comparators()
        L = ctypes.CDLL(str(path))
        L.sgc_plain_tables_steps.restype = c_int32
        L.sgc_plain_tables_steps.argtypes = [c_void_p, c_int64, c_void_p, c_void_p, c_void_p, c_int32, c_void_p,
                                             c_int32, c_void_p, POINTER(c_double), POINTER(c_double)]
        L.sgc_serial_replay.restype = c_int32
        L.sgc_serial_replay.argtypes = [c_void_p, c_void_p, c_int64, c_void_p, c_int32, c_void_p, c_void_p,
                                        c_void_p, POINTER(c_double), c_int32, POINTER(c_int64)]
        _lib = L
    return _lib


def handles(tables) -> np.ndarray:
    """Array of the tables' C handles (index = table id)."""
    return np.array([t._h.value for t in tables], dtype=np.uint64)


def plain_tables_steps(tables, keys, queries, offsets: np.ndarray, key_bytes: int, out_flags, steps: int,
                       stream) -> tuple[float, float]:
    """clear + insert + contains per table, `steps` times, from a C++ loop: (GPU ms, host ms) per step."""
    h = handles(tables)
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    g, w = c_double(), c_double()
    N.check(load().sgc_plain_tables_steps(c_void_p(h.ctypes.data), len(tables), c_void_p(keys.data_ptr()),
                                          c_void_p(queries.data_ptr()), c_void_p(off.ctypes.data), key_bytes,
                                          c_void_p(out_flags.data_ptr()), steps, c_void_p(stream.cuda_stream),
                                          ctypes.byref(g), ctypes.byref(w)), "plain_tables_steps")
    return g.value, w.value


def serial_replay(tables, requests, arrivals=None, sync_each: bool = True, stream=None, kernel_times=False,
                  grow_kind: int | None = None):
    """One request at a time on plain tables from a C++ loop.  requests: sequence of N.sg_request.  With
    grow_kind (the tables' kind) the loop grows a table before an insert as the server does.  Returns
    (latencies_us or None, kernel_us or None, wall_s, rehashes)."""
    import torch
    n = len(requests)
    arr = (N.sg_request * n)(*requests)
    h = handles(tables)
    lat = np.zeros(n, np.float64)
    ker = np.zeros(n, np.float32) if kernel_times else None
    arrv = None if arrivals is None else np.ascontiguousarray(arrivals, dtype=np.float64)
    if arrv is not None and len(arrv) < n:
        raise ValueError("one arrival time per request expected")
    wall = c_double()
    grown = c_int64()
    st = stream if stream is not None else torch.cuda.current_stream()
    N.check(load().sgc_serial_replay(c_void_p(h.ctypes.data), ctypes.cast(arr, c_void_p), n,
                                     None if arrv is None else c_void_p(arrv.ctypes.data), int(bool(sync_each)),
                                     c_void_p(st.cuda_stream), c_void_p(lat.ctypes.data),
                                     None if ker is None else c_void_p(ker.ctypes.data), ctypes.byref(wall),
                                     -1 if grow_kind is None else int(grow_kind), ctypes.byref(grown)),
            "serial_replay")
    return (lat if sync_each else None), ker, wall.value, grown.value

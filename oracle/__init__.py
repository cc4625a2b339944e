"""Oracle -- test infrastructure only (the checker, never the thing measured or shipped).

Two CPU implementations with one interface:

* ``PortTable`` / ``port_*``: the plain-C restatement in ``oracle/port.c``.
* ``RefTable`` / ``ref_*``: the reference library itself (stdgpu 1.3.0, OpenMP
  backend) through ``oracle/ref_driver.cpp``; available where
  ``oracle/build_oracle.py`` could build ``oracle/_ref/libsgref.so``.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py`` (its CPU-baseline
leg and its reference arm) may import this package.
"""

from __future__ import annotations

import ctypes
from ctypes import POINTER, byref, c_int, c_int64, c_uint8, c_void_p
from pathlib import Path

import numpy as np

from . import build_oracle

HERE = Path(__file__).resolve().parent

# container kinds, numbered as in include/stdgpu_gb300.h
SET_U32, SET_U64, MAP_U64_U32, MAP_U64_U64, MAP_U32_U32, MAP_U32_U64 = range(6)
KEY_DTYPE = {SET_U32: np.uint32, SET_U64: np.uint64, MAP_U64_U32: np.uint64, MAP_U64_U64: np.uint64,
             MAP_U32_U32: np.uint32, MAP_U32_U64: np.uint32}
VAL_DTYPE = {SET_U32: None, SET_U64: None, MAP_U64_U32: np.uint32, MAP_U64_U64: np.uint64,
             MAP_U32_U32: np.uint32, MAP_U32_U64: np.uint64}

# A custom key type with a user hash, as the reference's users write them: 3 x int16 coordinates hashed by
# the spatial hash of Teschner et al. (2003) (oracle/ref_driver.cpp; the reference's tests use this pair,
# tests/stdgpu/unordered_map.inc:178-206).  Only RefTable takes these kinds; the port and the GPU tables
# store such a key as its zero-padded 8-byte word with the hash passed per key.
SET_VEC3I16, MAP_VEC3I16_U32 = 6, 7
VEC3I16 = np.dtype([("x", "<i2"), ("y", "<i2"), ("z", "<i2")])
KEY_DTYPE[SET_VEC3I16] = VEC3I16
KEY_DTYPE[MAP_VEC3I16_U32] = VEC3I16
VAL_DTYPE[SET_VEC3I16] = None
VAL_DTYPE[MAP_VEC3I16_U32] = np.uint32
# the word-keyed kinds holding them (8-byte key words)
WORD_KIND = {SET_VEC3I16: SET_U64, MAP_VEC3I16_U32: MAP_U64_U32}

# A 12-byte key (3 x int32, with a user-declared destructor in oracle/ref_driver.cpp, the shape of the
# reference's nontrivial-type tests) under the same spatial hash; the GPU side holds it in the wide tables
# of the C++ API (16-byte key words).  Only RefTable takes these kinds.
SET_VEC3I32, MAP_VEC3I32_U64 = 8, 9
VEC3I32 = np.dtype([("x", "<i4"), ("y", "<i4"), ("z", "<i4")])
KEY_DTYPE[SET_VEC3I32] = VEC3I32
KEY_DTYPE[MAP_VEC3I32_U64] = VEC3I32
VAL_DTYPE[SET_VEC3I32] = None
VAL_DTYPE[MAP_VEC3I32_U64] = np.uint64


def vec3i16_words(keys: np.ndarray) -> np.ndarray:
    """Object bytes of each 6-byte key, zero-padded to a little-endian 64-bit word."""
    k = np.ascontiguousarray(keys, dtype=VEC3I16)
    w = np.zeros(len(k), np.uint64)
    w.view(np.uint8).reshape(-1, 8)[:, :6] = k.view(np.uint8).reshape(-1, 6)
    return w


def words_vec3i16(words: np.ndarray) -> np.ndarray:
    w = np.ascontiguousarray(words, dtype=np.uint64)
    k = np.zeros(len(w), VEC3I16)
    k.view(np.uint8).reshape(-1, 6)[:] = w.view(np.uint8).reshape(-1, 8)[:, :6]
    return k


def fibonacci_buckets(hashes: np.ndarray, bucket_count: int) -> np.ndarray:
    """The reference's fibonacci_hashing of each hash (src/stdgpu/impl/unordered_base_detail.cuh:56-85)."""
    h = np.ascontiguousarray(hashes, dtype=np.uint64)
    bits = int(bucket_count).bit_length() - 1
    if bits <= 0:
        return np.zeros(len(h), np.uint64)
    drop = np.uint64(64 - bits)
    with np.errstate(over="ignore"):
        return ((h ^ (h >> drop)) * np.uint64(11400714819323198485)) >> drop


def spatial_hash(keys: np.ndarray) -> np.ndarray:
    """(size_t(x) * 73856093) ^ (size_t(y) * 19349669) ^ (size_t(z) * 83492791), coordinates sign-extended;
    keys of VEC3I16 or VEC3I32."""
    k = np.ascontiguousarray(keys, dtype=keys.dtype if keys.dtype == VEC3I32 else VEC3I16)
    with np.errstate(over="ignore"):
        hx = k["x"].astype(np.int64).astype(np.uint64) * np.uint64(73856093)
        hy = k["y"].astype(np.int64).astype(np.uint64) * np.uint64(19349669)
        hz = k["z"].astype(np.int64).astype(np.uint64) * np.uint64(83492791)
    return hx ^ hy ^ hz

class SeqKeyTable:
    """Element-by-element restatement of the reference's bulk insert / erase / find for keys of any numpy
    record type (here the 12-byte VEC3I32): with one thread the reference processes a bulk call in input
    order, so an insert succeeds for the first copy of a key that is not stored yet
    (src/stdgpu/impl/unordered_base_detail.cuh:708-809, insert_value :996-1017) and an erase for the first
    copy of a stored key (:811-913, erase_from_key :1045-1066); a map keeps the value of the copy that was
    inserted.  Pure Python: small cases only."""

    def __init__(self, capacity: int, max_size: int):
        self.capacity = capacity
        self.max_size = max_size
        self.items: dict[bytes, object] = {}

    def insert(self, keys: np.ndarray, vals=None) -> np.ndarray:
        flags = np.zeros(len(keys), np.uint8)
        raw = np.ascontiguousarray(keys).view(np.uint8).reshape(len(keys), -1)
        for i in range(len(keys)):
            b = raw[i].tobytes()
            if b not in self.items and len(self.items) < self.max_size:
                self.items[b] = None if vals is None else vals[i]
                flags[i] = 1
        return flags

    def erase(self, keys: np.ndarray) -> np.ndarray:
        flags = np.zeros(len(keys), np.uint8)
        raw = np.ascontiguousarray(keys).view(np.uint8).reshape(len(keys), -1)
        for i in range(len(keys)):
            b = raw[i].tobytes()
            if b in self.items:
                del self.items[b]
                flags[i] = 1
        return flags

    def find(self, keys: np.ndarray):
        raw = np.ascontiguousarray(keys).view(np.uint8).reshape(len(keys), -1)
        found = np.array([raw[i].tobytes() in self.items for i in range(len(keys))], np.uint8)
        vals = [self.items.get(raw[i].tobytes()) for i in range(len(keys))]
        return vals, found

    def size(self) -> int:
        return len(self.items)

    def keys(self, dtype) -> np.ndarray:
        buf = b"".join(self.items.keys())
        return np.frombuffer(buf, dtype=dtype).copy() if buf else np.zeros(0, dtype)


_port = None
_ref = None


def _p(a: np.ndarray | None) -> c_void_p:
    return c_void_p(0) if a is None else c_void_p(a.ctypes.data)


def port_lib() -> ctypes.CDLL:
    global _port
    if _port is None:
        _port = ctypes.CDLL(str(build_oracle.build_port()))
        L = _port
        L.port_create.restype = c_void_p
        L.port_create.argtypes = [c_int64]
        L.port_destroy.argtypes = [c_void_p]
        for f in ("port_size", "port_bucket_count", "port_max_size", "port_excess_used", "port_range", "port_bucket",
                  "port_bucket_size", "port_fibonacci_hashing", "port_expected_collisions",
                  "port_vector_push_back", "port_deque_ops", "port_bitset_count"):
            getattr(L, f).restype = c_int64
        L.port_size.argtypes = [c_void_p]
        L.port_bucket_count.argtypes = [c_void_p]
        L.port_max_size.argtypes = [c_void_p]
        L.port_excess_used.argtypes = [c_void_p]
        L.port_bucket.argtypes = [c_void_p, ctypes.c_uint64]
        L.port_bucket_size.argtypes = [c_void_p, c_int64]
        L.port_fibonacci_hashing.argtypes = [ctypes.c_uint64, c_int64]
        L.port_expected_collisions.argtypes = [c_int64, c_int64]
        L.port_geometry.argtypes = [c_int64, POINTER(c_int64), POINTER(c_int64), POINTER(c_int64)]
        L.port_insert_bulk.argtypes = [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]
        L.port_erase_bulk.argtypes = [c_void_p, c_void_p, c_int64, c_void_p]
        L.port_find_bulk.argtypes = [c_void_p, c_void_p, c_int64, c_void_p, c_void_p]
        L.port_clear.argtypes = [c_void_p]
        L.port_valid.argtypes = [c_void_p]
        L.port_range.argtypes = [c_void_p, c_void_p, c_void_p]
        L.port_vector_push_back.argtypes = [c_int64, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]
        L.port_deque_ops.argtypes = [c_int64, c_void_p, c_int64, c_void_p, c_void_p, c_int64, c_void_p, c_void_p,
                                     c_void_p]
        L.port_bitset_count.argtypes = [c_void_p, c_int64]
        L.port_insert_bulk_h.argtypes = [c_void_p, c_void_p, c_void_p, c_void_p, c_int64, c_void_p]
        L.port_erase_bulk_h.argtypes = [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]
        L.port_find_bulk_h.argtypes = [c_void_p, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]
    return _port


def ref_available() -> bool:
    try:
        ref_lib()
        return True
    except (OSError, RuntimeError):
        return False


def ref_lib() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        so = build_oracle.build_reference()
        if so is None:
            raise RuntimeError("reference library not available (no staged reference tree)")
        L = ctypes.CDLL(str(so))
        L.sgref_create.restype = c_void_p
        L.sgref_create.argtypes = [c_int, c_int64]
        L.sgref_destroy.argtypes = [c_void_p]
        L.sgref_insert.argtypes = [c_void_p, c_void_p, c_void_p, c_int64]
        L.sgref_insert_flags.argtypes = [c_void_p, c_void_p, c_void_p, c_int64, c_void_p]
        L.sgref_erase.argtypes = [c_void_p, c_void_p, c_int64]
        L.sgref_erase_flags.argtypes = [c_void_p, c_void_p, c_int64, c_void_p]
        L.sgref_find.argtypes = [c_void_p, c_void_p, c_int64, c_void_p, c_void_p]
        L.sgref_contains.argtypes = [c_void_p, c_void_p, c_int64, c_void_p]
        L.sgref_size.restype = c_int64
        L.sgref_size.argtypes = [c_void_p]
        L.sgref_valid.argtypes = [c_void_p]
        L.sgref_clear.argtypes = [c_void_p]
        L.sgref_range.restype = c_int64
        L.sgref_range.argtypes = [c_void_p, c_void_p, c_void_p]
        L.sgref_bucket.restype = c_int64
        L.sgref_bucket.argtypes = [c_void_p, c_void_p]
        L.sgref_geometry.argtypes = [c_void_p, POINTER(c_int64), POINTER(c_int64)]
        L.sgref_set_threads.argtypes = [c_int]
        L.sgref_vector_push_back.restype = c_int64
        L.sgref_vector_push_back.argtypes = [c_int64, c_void_p, c_void_p, c_int64, c_void_p, c_void_p]
        L.sgref_deque_ops.restype = c_int64
        L.sgref_deque_ops.argtypes = [c_int64, c_void_p, c_int64, c_void_p, c_void_p, c_int64, c_void_p, c_void_p,
                                      c_void_p]
        L.sgref_bitset_count.restype = c_int64
        L.sgref_bitset_count.argtypes = [c_void_p, c_int64]
        L.sgref_std_unordered_map_run.restype = ctypes.c_double
        L.sgref_std_unordered_map_run.argtypes = [c_void_p, c_void_p, c_int64, c_void_p, c_int64, c_void_p, c_int64,
                                                  POINTER(c_int64), POINTER(ctypes.c_uint64), POINTER(c_int64)]
        _ref = L
    return _ref


def ref_std_unordered_map(keys, vals, queries, erase) -> tuple[float, int, int, int]:
    """std::unordered_map<uint64_t, uint32_t> in one thread over the same insert / find / erase sequence:
    (wall seconds, hits, sum of the values found, final size)."""
    k = np.ascontiguousarray(keys, dtype=np.uint64)
    v = np.ascontiguousarray(vals, dtype=np.uint32)
    q = np.ascontiguousarray(queries, dtype=np.uint64)
    e = np.ascontiguousarray(erase, dtype=np.uint64)
    hits, vsum, size = c_int64(), ctypes.c_uint64(), c_int64()
    secs = ref_lib().sgref_std_unordered_map_run(_p(k), _p(v), len(k), _p(q), len(q), _p(e), len(e), byref(hits),
                                                  byref(vsum), byref(size))
    return float(secs), hits.value, vsum.value, size.value


def ref_set_threads(n: int) -> None:
    ref_lib().sgref_set_threads(int(n))


def ref_max_threads() -> int:
    return int(ref_lib().sgref_max_threads())


class _TableBase:
    """Common numpy-facing surface of the two oracles."""

    kind: int

    def _keys(self, keys) -> np.ndarray:
        return np.ascontiguousarray(keys, dtype=KEY_DTYPE[self.kind])

    def _vals(self, vals, n) -> np.ndarray | None:
        vd = VAL_DTYPE[self.kind]
        if vd is None:
            return None
        if vals is None:
            return np.zeros(n, dtype=vd)
        return np.ascontiguousarray(vals, dtype=vd)


class PortTable(_TableBase):
    """unordered_set / unordered_map restated in C (oracle/port.c); keys and values carried as uint64."""

    def __init__(self, kind: int, capacity: int):
        self.kind = kind
        self.L = port_lib()
        self.h = c_void_p(self.L.port_create(int(capacity)))

    def close(self):
        if self.h:
            self.L.port_destroy(self.h)
            self.h = c_void_p(0)

    __del__ = close

    # hashes (optional, uint64 per key): Hash(key) of a custom key type; keys are then the key words
    def insert(self, keys, vals=None, flags: bool = False, hashes=None):
        k = self._keys(keys).astype(np.uint64)
        v = self._vals(vals, len(k))
        v64 = None if v is None else v.astype(np.uint64)
        f = np.zeros(len(k), np.uint8) if flags else None
        if hashes is None:
            self.L.port_insert_bulk(self.h, _p(k), _p(v64), len(k), _p(f))
        else:
            h = np.ascontiguousarray(hashes, dtype=np.uint64)
            self.L.port_insert_bulk_h(self.h, _p(k), _p(h), _p(v64), len(k), _p(f))
        return f

    def erase(self, keys, flags: bool = False, hashes=None):
        k = self._keys(keys).astype(np.uint64)
        f = np.zeros(len(k), np.uint8) if flags else None
        if hashes is None:
            self.L.port_erase_bulk(self.h, _p(k), len(k), _p(f))
        else:
            h = np.ascontiguousarray(hashes, dtype=np.uint64)
            self.L.port_erase_bulk_h(self.h, _p(k), _p(h), len(k), _p(f))
        return f

    def find(self, keys, hashes=None):
        k = self._keys(keys).astype(np.uint64)
        v = np.zeros(len(k), np.uint64)
        f = np.zeros(len(k), np.uint8)
        if hashes is None:
            self.L.port_find_bulk(self.h, _p(k), len(k), _p(v), _p(f))
        else:
            h = np.ascontiguousarray(hashes, dtype=np.uint64)
            self.L.port_find_bulk_h(self.h, _p(k), _p(h), len(k), _p(v), _p(f))
        vd = VAL_DTYPE[self.kind]
        return (v.astype(vd) if vd is not None else None), f

    def contains(self, keys):
        return self.find(keys)[1]

    def size(self) -> int:
        return int(self.L.port_size(self.h))

    def excess_used(self) -> int:
        return int(self.L.port_excess_used(self.h))

    def valid(self) -> bool:
        return bool(self.L.port_valid(self.h))

    def clear(self):
        self.L.port_clear(self.h)

    def bucket(self, key: int) -> int:
        return int(self.L.port_bucket(self.h, int(key)))

    def bucket_size(self, n: int) -> int:
        return int(self.L.port_bucket_size(self.h, int(n)))

    def geometry(self) -> tuple[int, int]:
        return int(self.L.port_bucket_count(self.h)), int(self.L.port_max_size(self.h))

    def range(self):
        n_max = self.geometry()[1]
        k = np.zeros(n_max, np.uint64)
        v = np.zeros(n_max, np.uint64)
        n = int(self.L.port_range(self.h, _p(k), _p(v)))
        vd = VAL_DTYPE[self.kind]
        return k[:n].astype(KEY_DTYPE[self.kind]), (v[:n].astype(vd) if vd is not None else None)


class RefTable(_TableBase):
    """The reference's own unordered_set / unordered_map (OpenMP backend) behind the same surface."""

    def __init__(self, kind: int, capacity: int):
        self.kind = kind
        self.L = ref_lib()
        self.h = c_void_p(self.L.sgref_create(kind, int(capacity)))
        if not self.h:
            raise ValueError("unknown kind")

    def close(self):
        if self.h:
            self.L.sgref_destroy(self.h)
            self.h = c_void_p(0)

    __del__ = close

    def insert(self, keys, vals=None, flags: bool = False):
        k = self._keys(keys)
        v = self._vals(vals, len(k))
        if flags:
            f = np.zeros(len(k), np.uint8)
            self.L.sgref_insert_flags(self.h, _p(k), _p(v), len(k), _p(f))
            return f
        self.L.sgref_insert(self.h, _p(k), _p(v), len(k))
        return None

    def erase(self, keys, flags: bool = False):
        k = self._keys(keys)
        if flags:
            f = np.zeros(len(k), np.uint8)
            self.L.sgref_erase_flags(self.h, _p(k), len(k), _p(f))
            return f
        self.L.sgref_erase(self.h, _p(k), len(k))
        return None

    def find(self, keys):
        k = self._keys(keys)
        vd = VAL_DTYPE[self.kind]
        v = np.zeros(len(k), vd) if vd is not None else None
        f = np.zeros(len(k), np.uint8)
        self.L.sgref_find(self.h, _p(k), len(k), _p(v), _p(f))
        return v, f

    def contains(self, keys):
        k = self._keys(keys)
        f = np.zeros(len(k), np.uint8)
        self.L.sgref_contains(self.h, _p(k), len(k), _p(f))
        return f

    def size(self) -> int:
        return int(self.L.sgref_size(self.h))

    def valid(self) -> bool:
        return bool(self.L.sgref_valid(self.h))

    def clear(self):
        self.L.sgref_clear(self.h)

    def bucket(self, key: int) -> int:
        k = np.array([key], dtype=KEY_DTYPE[self.kind])
        return int(self.L.sgref_bucket(self.h, _p(k)))

    def bucket_of(self, key) -> int:
        """bucket() of one key of any key type (a numpy scalar or record)."""
        k = np.array([key], dtype=KEY_DTYPE[self.kind])
        return int(self.L.sgref_bucket(self.h, _p(k)))

    def geometry(self) -> tuple[int, int]:
        b, m = c_int64(), c_int64()
        self.L.sgref_geometry(self.h, byref(b), byref(m))
        return b.value, m.value

    def range(self):
        n_max = self.geometry()[1]
        k = np.zeros(n_max, KEY_DTYPE[self.kind])
        vd = VAL_DTYPE[self.kind]
        v = np.zeros(n_max, vd) if vd is not None else None
        n = int(self.L.sgref_range(self.h, _p(k), _p(v)))
        return k[:n], (v[:n] if v is not None else None)


def port_geometry(capacity: int) -> tuple[int, int, int]:
    b, e, t = c_int64(), c_int64(), c_int64()
    port_lib().port_geometry(int(capacity), byref(b), byref(e), byref(t))
    return b.value, e.value, t.value


def port_fibonacci_hashing(h: int, bucket_count: int) -> int:
    return int(port_lib().port_fibonacci_hashing(int(h), int(bucket_count)))


def port_vector_push_back(capacity: int, values, pred=None):
    """Returns (size, pushed flags, contents)."""
    v = np.ascontiguousarray(values, dtype=np.uint64)
    p = None if pred is None else np.ascontiguousarray(pred, dtype=np.uint8)
    pushed = np.zeros(len(v), np.uint8)
    out = np.zeros(max(capacity, 1), np.uint64)
    n = int(port_lib().port_vector_push_back(int(capacity), _p(v), _p(p), len(v), _p(pushed), _p(out)))
    return n, pushed, out[:n]


def ref_vector_push_back(capacity: int, values, pred=None):
    v = np.ascontiguousarray(values, dtype=np.uint32)
    p = None if pred is None else np.ascontiguousarray(pred, dtype=np.uint8)
    pushed = np.zeros(len(v), np.uint8)
    out = np.zeros(max(capacity, 1), np.uint32)
    n = int(ref_lib().sgref_vector_push_back(int(capacity), _p(v), _p(p), len(v), _p(pushed), _p(out)))
    return n, pushed, out[:n]


def port_deque_ops(capacity: int, init, is_push, values):
    """Returns (size, popped, ok, remaining front-to-back)."""
    i = np.ascontiguousarray(init, dtype=np.uint64)
    ip = np.ascontiguousarray(is_push, dtype=np.uint8)
    v = np.ascontiguousarray(values, dtype=np.uint64)
    popped = np.zeros(len(v), np.uint64)
    ok = np.zeros(len(v), np.uint8)
    rem = np.zeros(max(capacity, 1), np.uint64)
    n = int(port_lib().port_deque_ops(int(capacity), _p(i), len(i), _p(ip), _p(v), len(v), _p(popped), _p(ok),
                                      _p(rem)))
    return n, popped, ok, rem[:n]


def ref_deque_ops(capacity: int, init, is_push, values):
    i = np.ascontiguousarray(init, dtype=np.uint64)
    ip = np.ascontiguousarray(is_push, dtype=np.uint8)
    v = np.ascontiguousarray(values, dtype=np.uint64)
    popped = np.zeros(len(v), np.uint64)
    ok = np.zeros(len(v), np.uint8)
    rem = np.zeros(max(capacity, 1), np.uint64)
    n = int(ref_lib().sgref_deque_ops(int(capacity), _p(i), len(i), _p(ip), _p(v), len(v), _p(popped), _p(ok),
                                      _p(rem)))
    return n, popped, ok, rem[:n]


def port_bitset_count(words, nbits: int) -> int:
    w = np.ascontiguousarray(words, dtype=np.uint32)
    return int(port_lib().port_bitset_count(_p(w), int(nbits)))


def ref_bitset_count(words, nbits: int) -> int:
    w = np.ascontiguousarray(words, dtype=np.uint32)
    return int(ref_lib().sgref_bitset_count(_p(w), int(nbits)))

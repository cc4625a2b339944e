"""Python host mirror of the reference containers on the hot path.

Names and argument meaning follow the reference's C++ API
(``stdgpu::unordered_map`` / ``unordered_set`` / ``vector`` / ``deque`` /
``bitset::count``, src/stdgpu/*.cuh); every call goes through the C ABI of the
native library (``include/stdgpu_gb300.h``).  Device buffers are torch CUDA
tensors used purely as memory: keys and values are 4- or 8-byte integers and
are passed bit for bit (an int64 tensor carries uint64 keys).
"""

from __future__ import annotations

import ctypes
from ctypes import byref, c_int32, c_int64, c_void_p

import torch

from . import _native as N

_KEY_BYTES = {N.SET_U32: 4, N.SET_U64: 8, N.MAP_U64_U32: 8, N.MAP_U64_U64: 8, N.MAP_U32_U32: 4, N.MAP_U32_U64: 4}
_MAPPED_BYTES = {N.SET_U32: 0, N.SET_U64: 0, N.MAP_U64_U32: 4, N.MAP_U64_U64: 8, N.MAP_U32_U32: 4,
                 N.MAP_U32_U64: 8}
_INT_DTYPE = {4: torch.int32, 8: torch.int64}

KINDS = {("u32", None): N.SET_U32, ("u64", None): N.SET_U64, ("u64", "u32"): N.MAP_U64_U32,
         ("u64", "u64"): N.MAP_U64_U64, ("u32", "u32"): N.MAP_U32_U32, ("u32", "u64"): N.MAP_U32_U64}


def _stream(stream) -> c_void_p:
    if stream is None:
        stream = torch.cuda.current_stream()
    return c_void_p(stream.cuda_stream)


def _ptr(t: torch.Tensor | None) -> c_void_p:
    if t is None:
        return c_void_p(0)
    if not t.is_cuda:
        raise ValueError("device tensor expected")
    if not t.is_contiguous():
        raise ValueError("contiguous tensor expected")
    return c_void_p(t.data_ptr())


def _as_bits(t: torch.Tensor, nbytes: int, what: str) -> torch.Tensor:
    if t.element_size() != nbytes:
        raise ValueError(f"{what}: {nbytes}-byte elements expected, got {t.dtype}")
    return t.contiguous()


def _hptr(t: torch.Tensor | None) -> c_void_p:
    if t is None:
        return c_void_p(0)
    if t.is_cuda:
        raise ValueError("host tensor expected")
    if not t.is_contiguous():
        raise ValueError("contiguous tensor expected")
    return c_void_p(t.data_ptr())


class stager:
    """Pipeline for table calls on host tensors (sg_stager_*): chunks of `chunk_elems` elements are copied
    in through `buffers` device staging buffers while earlier chunks' kernels run, and results are copied
    back while later chunks run.  Host tensors should be pinned (``tensor.pin_memory()``) for overlap."""

    def __init__(self, chunk_elems: int = 1 << 22, buffers: int = 4):
        h = c_void_p()
        N.check(N.load().sg_stager_create(int(chunk_elems), int(buffers), byref(h)), "stager::create")
        self._h = h
        self.chunk_elems = int(chunk_elems)
        self.buffers = int(buffers)

    def set_inputs_ready(self, ready: bool = True) -> None:
        """Uploads start when a call is made, not after the stream's earlier work (sg_stager_set_inputs_ready);
        the caller vouches that no earlier work writes the call's host inputs."""
        N.check(N.load().sg_stager_set_inputs_ready(self._h, int(bool(ready))), "stager::set_inputs_ready")

    def close(self) -> None:
        if self._h:
            N.check(N.load().sg_stager_destroy(self._h), "stager::destroy")
            self._h = c_void_p(0)


_default_stagers: dict[int, stager] = {}


def default_stager() -> stager:
    """One stager per device, created on first use by a call on host tensors."""
    d = torch.cuda.current_device()
    if d not in _default_stagers:
        _default_stagers[d] = stager()
    return _default_stagers[d]


def _host_out(n: int, dtype) -> torch.Tensor:
    return torch.empty(n, dtype=dtype).pin_memory()


class unordered_base:
    """Shared implementation of unordered_set / unordered_map (src/stdgpu/impl/unordered_base.cuh:56-583)."""

    def __init__(self, handle: int, kind: int, custom_hash: bool = False):
        self._h = c_void_p(handle)
        self.kind = kind
        # custom key types: keys are key words, and every bulk call takes hashes=Hash(key) per key
        self.custom_hash = custom_hash
        self.key_bytes = _KEY_BYTES[kind]
        self.mapped_bytes = _MAPPED_BYTES[kind]
        g = N.sg_geometry()
        N.check(N.load().sg_unordered_geometry(self._h, byref(g)), "geometry")
        self._geom = g

    # ---- create / destroy: unordered_base_detail.cuh:1254-1348
    @classmethod
    def _create(cls, kind: int, capacity: int, stream=None, custom_hash: bool = False):
        lib = N.load()
        h = c_void_p()
        create = lib.sg_unordered_create_hashed if custom_hash else lib.sg_unordered_create
        N.check(create(kind, int(capacity), _stream(stream), byref(h)), "createDeviceObject")
        return cls(h.value, kind, custom_hash)

    def _hashes(self, hashes, n: int) -> c_void_p:
        if not self.custom_hash:
            if hashes is not None:
                raise ValueError("hashes are for tables created with custom_hash=True")
            return c_void_p(0)
        if hashes is None or hashes.numel() != n or hashes.element_size() != 8:
            raise ValueError("a custom-hash table needs one 64-bit hash per key")
        return _ptr(hashes.contiguous())

    @staticmethod
    def destroyDeviceObject(obj: "unordered_base") -> None:
        if obj._h:
            N.check(N.load().sg_unordered_destroy(obj._h), "destroyDeviceObject")
            obj._h = c_void_p(0)

    # ---- geometry: unordered_base_detail.cuh:1134-1176
    def bucket_count(self) -> int:
        return self._geom.bucket_count

    def max_size(self) -> int:
        return self._geom.max_size

    def max_load_factor(self) -> float:
        return 1.0

    def geometry(self) -> N.sg_geometry:
        return self._geom

    def load_factor(self, stream=None) -> float:
        # float division as in unordered_base_detail.cuh:1155-1160
        import numpy as np
        return float(np.float32(self.size(stream)) / np.float32(self.bucket_count()))

    def bucket_of_hash(self, hash_value: int) -> int:
        """bucket() of a key whose Hash is hash_value (custom key types)."""
        out = c_int64()
        N.check(N.load().sg_unordered_bucket_of_hash(self._h, int(hash_value) & (2**64 - 1), byref(out)), "bucket")
        return out.value

    def bucket(self, key: int) -> int:
        kb = self.key_bytes
        buf = (ctypes.c_uint32 if kb == 4 else ctypes.c_uint64)(int(key) & ((1 << (8 * kb)) - 1))
        out = c_int64()
        N.check(N.load().sg_unordered_bucket(self._h, ctypes.cast(byref(buf), c_void_p), byref(out)), "bucket")
        return out.value

    # ---- bulk operations
    # Each accepts device tensors (stream-ordered, asynchronous) or host tensors; with host tensors the call
    # streams through a stager (`stager=`, else the device's default one) and returns after the stream has
    # finished it, so host inputs may be reused and host outputs read at once.
    def _host_done(self, stream) -> None:
        (stream if stream is not None else torch.cuda.current_stream()).synchronize()

    def insert(self, keys: torch.Tensor, mapped: torch.Tensor | None = None, *, flags: torch.Tensor | None = None,
               stream=None, stager: "stager | None" = None, hashes: torch.Tensor | None = None) -> None:
        """insert(begin, end) over keys (+ mapped values for maps): unordered_base_detail.cuh:996-1017."""
        keys = _as_bits(keys, self.key_bytes, "keys")
        if self.mapped_bytes:
            if mapped is None:
                raise ValueError("mapped values required for a map")
            mapped = _as_bits(mapped, self.mapped_bytes, "mapped")
        else:
            mapped = None
        if self.custom_hash:
            N.check(N.load().sg_unordered_insert_hashed(self._h, _ptr(keys), _ptr(mapped),
                                                        self._hashes(hashes, keys.numel()), keys.numel(), _ptr(flags),
                                                        _stream(stream)), "insert")
            return
        if not keys.is_cuda:
            st = stager or default_stager()
            N.check(N.load().sg_unordered_insert_kv_host(self._h, st._h, _hptr(keys), _hptr(mapped), keys.numel(),
                                                         _hptr(flags), _stream(stream)), "insert")
            self._host_done(stream)
            return
        N.check(N.load().sg_unordered_insert_kv(self._h, _ptr(keys), _ptr(mapped), keys.numel(), _ptr(flags),
                                                _stream(stream)), "insert")

    def insert_values(self, values: torch.Tensor, n: int, *, flags: torch.Tensor | None = None, stream=None) -> None:
        """insert(begin, end) over a value_type array (raw bytes, n elements of slot_bytes)."""
        if values.numel() * values.element_size() < n * self._geom.slot_bytes:
            raise ValueError("values buffer too small")
        N.check(N.load().sg_unordered_insert(self._h, _ptr(values), int(n), _ptr(flags), _stream(stream)), "insert")

    def erase(self, keys: torch.Tensor, *, flags: torch.Tensor | None = None, stream=None,
              stager: "stager | None" = None, hashes: torch.Tensor | None = None) -> None:
        """erase(begin, end): unordered_base_detail.cuh:1045-1066."""
        keys = _as_bits(keys, self.key_bytes, "keys")
        if self.custom_hash:
            N.check(N.load().sg_unordered_erase_hashed(self._h, _ptr(keys), self._hashes(hashes, keys.numel()),
                                                       keys.numel(), _ptr(flags), _stream(stream)), "erase")
            return
        if not keys.is_cuda:
            st = stager or default_stager()
            N.check(N.load().sg_unordered_erase_host(self._h, st._h, _hptr(keys), keys.numel(), _hptr(flags),
                                                     _stream(stream)), "erase")
            self._host_done(stream)
            return
        N.check(N.load().sg_unordered_erase(self._h, _ptr(keys), keys.numel(), _ptr(flags), _stream(stream)),
                "erase")

    def contains(self, keys: torch.Tensor, stream=None, stager: "stager | None" = None,
                 hashes: torch.Tensor | None = None) -> torch.Tensor:
        keys = _as_bits(keys, self.key_bytes, "keys")
        if self.custom_hash:
            out = torch.empty(keys.numel(), dtype=torch.uint8, device=keys.device)
            N.check(N.load().sg_unordered_contains_hashed(self._h, _ptr(keys), self._hashes(hashes, keys.numel()),
                                                          keys.numel(), _ptr(out), _stream(stream)), "contains")
            return out
        if not keys.is_cuda:
            st = stager or default_stager()
            out = _host_out(keys.numel(), torch.uint8)
            N.check(N.load().sg_unordered_contains_host(self._h, st._h, _hptr(keys), keys.numel(), _hptr(out),
                                                        _stream(stream)), "contains")
            self._host_done(stream)
            return out
        out = torch.empty(keys.numel(), dtype=torch.uint8, device=keys.device)
        N.check(N.load().sg_unordered_contains(self._h, _ptr(keys), keys.numel(), _ptr(out), _stream(stream)),
                "contains")
        return out

    def count(self, keys: torch.Tensor, stream=None, hashes: torch.Tensor | None = None) -> torch.Tensor:
        return self.contains(keys, stream, hashes=hashes)

    def find(self, keys: torch.Tensor, stream=None, stager: "stager | None" = None,
             hashes: torch.Tensor | None = None) -> tuple[torch.Tensor | None, torch.Tensor]:
        keys = _as_bits(keys, self.key_bytes, "keys")
        if self.custom_hash:
            found = torch.empty(keys.numel(), dtype=torch.uint8, device=keys.device)
            vals = None
            if self.mapped_bytes:
                vals = torch.zeros(keys.numel(), dtype=_INT_DTYPE[self.mapped_bytes], device=keys.device)
            N.check(N.load().sg_unordered_find_hashed(self._h, _ptr(keys), self._hashes(hashes, keys.numel()),
                                                      keys.numel(), _ptr(vals), _ptr(found), _stream(stream)), "find")
            return vals, found
        if not keys.is_cuda:
            st = stager or default_stager()
            found = _host_out(keys.numel(), torch.uint8)
            vals = _host_out(keys.numel(), _INT_DTYPE[self.mapped_bytes]) if self.mapped_bytes else None
            N.check(N.load().sg_unordered_find_host(self._h, st._h, _hptr(keys), keys.numel(), _hptr(vals),
                                                    _hptr(found), _stream(stream)), "find")
            self._host_done(stream)
            return vals, found
        found = torch.empty(keys.numel(), dtype=torch.uint8, device=keys.device)
        vals = None
        if self.mapped_bytes:
            vals = torch.zeros(keys.numel(), dtype=_INT_DTYPE[self.mapped_bytes], device=keys.device)
        N.check(N.load().sg_unordered_find(self._h, _ptr(keys), keys.numel(), _ptr(vals), _ptr(found),
                                           _stream(stream)), "find")
        return vals, found

    def size(self, stream=None) -> int:
        out = c_int64()
        N.check(N.load().sg_unordered_size(self._h, _stream(stream), byref(out)), "size")
        return out.value

    def status(self, stream=None) -> tuple[int, int, int]:
        """(status code, refused inserts since the last call, erased slots awaiting reuse)."""
        refused, tombs = c_int64(), c_int64()
        st = N.load().sg_unordered_status(self._h, _stream(stream), byref(refused), byref(tombs))
        N.check(st, "status", allow=(N.SG_ERR_FULL,))
        return st, refused.value, tombs.value

    def empty(self, stream=None) -> bool:
        return self.size(stream) == 0

    def full(self, stream=None) -> bool:
        return self.size(stream) == self.max_size()

    def clear(self, stream=None) -> None:
        N.check(N.load().sg_unordered_clear(self._h, _stream(stream)), "clear")

    def rehash(self, new_capacity: int, stream=None) -> None:
        """Move every element into storage for new_capacity (sg_unordered_rehash); synchronises."""
        N.check(N.load().sg_unordered_rehash(self._h, int(new_capacity), _stream(stream)), "rehash")
        g = N.sg_geometry()
        N.check(N.load().sg_unordered_geometry(self._h, byref(g)), "geometry")
        self._geom = g

    def save(self, path, stream=None) -> None:
        """Write a snapshot file (sg_unordered_save)."""
        N.check(N.load().sg_unordered_save(self._h, str(path).encode(), _stream(stream)), "save")

    @classmethod
    def load(cls, path, stream=None) -> "unordered_base":
        """Recreate a table from a snapshot file (sg_unordered_load)."""
        lib = N.load()
        h = c_void_p()
        N.check(lib.sg_unordered_load(str(path).encode(), _stream(stream), byref(h)), "load")
        v = N.sg_unordered_view()
        N.check(lib.sg_unordered_view_of(h, byref(v)), "load")
        hashed = c_int32()
        N.check(lib.sg_unordered_is_hashed(h, byref(hashed)), "load")
        return cls(h.value, v.kind, bool(hashed.value))

    INSERT_MODES = {"auto": 0, "direct": 1, "partitioned": 2}

    def set_insert_mode(self, mode: str) -> None:
        """Bulk-insert strategy: "auto", "direct" or "partitioned" (sg_unordered_set_insert_mode)."""
        N.check(N.load().sg_unordered_set_insert_mode(self._h, self.INSERT_MODES[mode]), "set_insert_mode")

    def set_excess_accounting(self, on: bool, stream=None) -> None:
        """The reference's refusal once its excess list is empty (sg_unordered_set_excess_accounting); on by
        default up to max_size() 2^20; only on an empty table."""
        N.check(N.load().sg_unordered_set_excess_accounting(self._h, int(bool(on)), _stream(stream)),
                "set_excess_accounting")

    def excess_used(self, stream=None) -> int:
        """Keys holding the reference's excess slots; -1 with the accounting off."""
        out = c_int64()
        N.check(N.load().sg_unordered_excess_used(self._h, _stream(stream), byref(out)), "excess_used")
        return out.value

    def valid(self, stream=None) -> bool:
        out = c_int32()
        N.check(N.load().sg_unordered_valid(self._h, _stream(stream), byref(out)), "valid")
        return bool(out.value)

    def device_range(self, stream=None) -> torch.Tensor:
        """Slot indices of all stored elements (device_range(): unordered_base_detail.cuh:160-208)."""
        out = torch.empty(self.max_size() + 2, dtype=torch.int32, device="cuda")
        n = c_int64()
        N.check(N.load().sg_unordered_device_range(self._h, _ptr(out), _stream(stream), byref(n)), "device_range")
        return out[: n.value]

    def range_copy(self, stream=None) -> tuple[torch.Tensor, torch.Tensor | None]:
        """(keys, mapped) of all stored elements, in slot order."""
        cap = self.max_size() + 2
        keys = torch.empty(cap, dtype=_INT_DTYPE[self.key_bytes], device="cuda")
        vals = torch.empty(cap, dtype=_INT_DTYPE[self.mapped_bytes], device="cuda") if self.mapped_bytes else None
        n = c_int64()
        N.check(N.load().sg_unordered_range_copy(self._h, _ptr(keys), _ptr(vals), _stream(stream), byref(n)),
                "range_copy")
        return keys[: n.value], (vals[: n.value] if vals is not None else None)

    def view(self) -> N.sg_unordered_view:
        v = N.sg_unordered_view()
        N.check(N.load().sg_unordered_view_of(self._h, byref(v)), "view")
        return v


class unordered_set(unordered_base):
    """stdgpu::unordered_set<Key> for Key = uint32_t / uint64_t (src/stdgpu/unordered_set.cuh:61-65)."""

    @classmethod
    def createDeviceObject(cls, capacity: int, key: str = "u64", stream=None,
                           custom_hash: bool = False) -> "unordered_set":
        return cls._create(KINDS[(key, None)], capacity, stream, custom_hash)


class unordered_map(unordered_base):
    """stdgpu::unordered_map<Key, T> for 4/8-byte integer Key and T (src/stdgpu/unordered_map.cuh:70-75)."""

    @classmethod
    def createDeviceObject(cls, capacity: int, key: str = "u64", mapped: str = "u32",
                           stream=None, custom_hash: bool = False) -> "unordered_map":
        return cls._create(KINDS[(key, mapped)], capacity, stream, custom_hash)


_allocator_callbacks = None


def use_torch_allocator(enable: bool = True) -> None:
    """Route the device storage of every container through PyTorch's caching allocator
    (sg_set_device_allocator), or back to cudaMalloc / cudaFree.  Only while no container is alive."""
    global _allocator_callbacks
    lib = N.load()
    if not enable:
        N.check(lib.sg_set_device_allocator(None, None, None), "set_device_allocator")
        _allocator_callbacks = None
        return
    alloc_t = ctypes.CFUNCTYPE(c_void_p, ctypes.c_size_t, c_void_p)
    free_t = ctypes.CFUNCTYPE(None, c_void_p, c_void_p)

    def alloc(nbytes, _ctx):
        try:
            return torch.cuda.caching_allocator_alloc(int(nbytes))
        except RuntimeError:
            return None

    def release(ptr, _ctx):
        torch.cuda.caching_allocator_delete(ptr)

    callbacks = (alloc_t(alloc), free_t(release))
    N.check(lib.sg_set_device_allocator(ctypes.cast(callbacks[0], c_void_p), ctypes.cast(callbacks[1], c_void_p),
                                        None), "set_device_allocator")
    _allocator_callbacks = callbacks  # the C function pointers must outlive their use


def live_device_allocations() -> int:
    return int(N.load().sg_live_device_allocations())


def geometry_for(kind: int, capacity: int) -> N.sg_geometry:
    g = N.sg_geometry()
    N.check(N.load().sg_unordered_geometry_for(kind, int(capacity), byref(g)), "geometry_for")
    return g


class table_batch:
    """Many independent unordered_set / unordered_map objects of one kind in one device arena.

    Operations take the keys of all tables concatenated with per-table offsets (a device int64 tensor
    of n_tables + 1 entries) and run as one persistent launch; a sequence of them can be captured in a
    CUDA graph.  No counterpart in the reference: it batches what the reference does with one
    createDeviceObject and one bulk call per table.
    """

    def __init__(self, handle: int, kind: int, n_tables: int):
        self._h = c_void_p(handle)
        self.kind = kind
        self.n_tables = n_tables
        self.key_bytes = _KEY_BYTES[kind]
        self.mapped_bytes = _MAPPED_BYTES[kind]

    @classmethod
    def createDeviceObjects(cls, capacities, key: str = "u64", mapped: str | None = None,
                            stream=None, tuning: dict | None = None) -> "table_batch":
        import numpy as np
        kind = KINDS[(key, mapped)]
        caps = np.ascontiguousarray(np.asarray(capacities, dtype=np.int64))
        h = c_void_p()
        N.check(N.load().sg_batch_create(kind, len(caps), c_void_p(caps.ctypes.data), _stream(stream), byref(h)),
                "batch::createDeviceObjects")
        b = cls(h.value, kind, len(caps))
        cfg = tuning if tuning is not None else load_batch_tuning()
        if cfg:
            b.configure(cfg["threads_per_block"], cfg["blocks_per_sm"], cfg["tiles_per_step"])
        return b

    @staticmethod
    def destroyDeviceObjects(b: "table_batch") -> None:
        if b._h:
            N.check(N.load().sg_batch_destroy(b._h), "batch::destroyDeviceObjects")
            b._h = c_void_p(0)

    def configure(self, threads_per_block: int, blocks_per_sm: int, tiles_per_step: int) -> None:
        N.check(N.load().sg_batch_configure(self._h, threads_per_block, blocks_per_sm, tiles_per_step),
                "batch::configure")

    def clear(self, stream=None) -> None:
        N.check(N.load().sg_batch_clear(self._h, _stream(stream)), "batch::clear")

    def insert(self, keys: torch.Tensor, offsets: torch.Tensor, mapped: torch.Tensor | None = None, *,
               flags: torch.Tensor | None = None, stream=None) -> None:
        keys = _as_bits(keys, self.key_bytes, "keys")
        if self.mapped_bytes:
            mapped = _as_bits(mapped, self.mapped_bytes, "mapped")
        N.check(N.load().sg_batch_insert_kv(self._h, _ptr(keys), _ptr(mapped if self.mapped_bytes else None),
                                            _ptr(_offsets(offsets)), _ptr(flags), _stream(stream)), "batch::insert")

    def erase(self, keys: torch.Tensor, offsets: torch.Tensor, *, flags: torch.Tensor | None = None,
              stream=None) -> None:
        keys = _as_bits(keys, self.key_bytes, "keys")
        N.check(N.load().sg_batch_erase(self._h, _ptr(keys), _ptr(_offsets(offsets)), _ptr(flags), _stream(stream)),
                "batch::erase")

    def contains(self, keys: torch.Tensor, offsets: torch.Tensor, out: torch.Tensor | None = None,
                 stream=None) -> torch.Tensor:
        keys = _as_bits(keys, self.key_bytes, "keys")
        if out is None:
            out = torch.empty(keys.numel(), dtype=torch.uint8, device=keys.device)
        N.check(N.load().sg_batch_contains(self._h, _ptr(keys), _ptr(_offsets(offsets)), _ptr(out),
                                           _stream(stream)), "batch::contains")
        return out

    def find(self, keys: torch.Tensor, offsets: torch.Tensor, stream=None):
        keys = _as_bits(keys, self.key_bytes, "keys")
        found = torch.empty(keys.numel(), dtype=torch.uint8, device=keys.device)
        vals = torch.zeros(keys.numel(), dtype=_INT_DTYPE[self.mapped_bytes], device=keys.device) \
            if self.mapped_bytes else None
        N.check(N.load().sg_batch_find(self._h, _ptr(keys), _ptr(_offsets(offsets)), _ptr(vals), _ptr(found),
                                       _stream(stream)), "batch::find")
        return vals, found

    def sizes(self, stream=None):
        import numpy as np
        out = np.zeros(self.n_tables, dtype=np.int64)
        N.check(N.load().sg_batch_sizes(self._h, _stream(stream), c_void_p(out.ctypes.data)), "batch::sizes")
        return out

    def view(self, table: int) -> N.sg_unordered_view:
        v = N.sg_unordered_view()
        N.check(N.load().sg_batch_view_of(self._h, int(table), byref(v)), "batch::view")
        return v

    def storage_bytes(self) -> int:
        b = c_int64()
        N.check(N.load().sg_batch_info(self._h, byref(b), None), "batch::info")
        return b.value


def _offsets(offsets: torch.Tensor) -> torch.Tensor:
    if offsets.dtype != torch.int64 or not offsets.is_cuda:
        raise ValueError("offsets: device int64 tensor of n_tables + 1 entries expected")
    return offsets.contiguous()


def load_batch_tuning() -> dict | None:
    """Launch shape chosen by stdgpu_gb300/autotune.py on a GB300, if recorded."""
    import json
    from pathlib import Path
    f = Path(__file__).resolve().parent / "tuning" / "batch.json"
    if f.exists():
        try:
            return json.loads(f.read_text())["best"]
        except (ValueError, KeyError):
            return None
    return None


class vector:
    """stdgpu::vector<T> (T = 4 or 8 bytes): push_back, size, clear (src/stdgpu/vector.cuh)."""

    def __init__(self, handle: int, elem_bytes: int, capacity: int):
        self._h = c_void_p(handle)
        self.elem_bytes = elem_bytes
        self._capacity = capacity

    @classmethod
    def createDeviceObject(cls, capacity: int, elem_bytes: int = 4) -> "vector":
        h = c_void_p()
        N.check(N.load().sg_vector_create(elem_bytes, int(capacity), byref(h)), "vector::createDeviceObject")
        return cls(h.value, elem_bytes, capacity)

    @staticmethod
    def destroyDeviceObject(v: "vector") -> None:
        if v._h:
            N.check(N.load().sg_vector_destroy(v._h), "vector::destroyDeviceObject")
            v._h = c_void_p(0)

    def capacity(self) -> int:
        return self._capacity

    def push_back(self, values: torch.Tensor, pred: torch.Tensor | None = None, *,
                  flags: torch.Tensor | None = None, stream=None) -> None:
        values = _as_bits(values, self.elem_bytes, "values")
        N.check(N.load().sg_vector_push_back(self._h, _ptr(values), _ptr(pred), values.numel(), _ptr(flags),
                                             _stream(stream)), "push_back")

    def size(self, stream=None) -> int:
        out = c_int64()
        N.check(N.load().sg_vector_size(self._h, _stream(stream), byref(out)), "vector::size")
        return out.value

    def clear(self, stream=None) -> None:
        N.check(N.load().sg_vector_clear(self._h, _stream(stream)), "vector::clear")

    def pop_back(self, n: int, stream=None) -> tuple[torch.Tensor, torch.Tensor]:
        """pop_back() n times; returns (values, ok): element i is the i-th from the back."""
        vals = torch.zeros(n, dtype=_INT_DTYPE[self.elem_bytes], device="cuda")
        ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
        N.check(N.load().sg_vector_pop_back(self._h, int(n), _ptr(vals), _ptr(ok), _stream(stream)), "pop_back")
        return vals, ok

    def insert(self, values: torch.Tensor, stream=None) -> None:
        """insert(device_end(), begin, end): append a range (refused whole when it does not fit)."""
        values = _as_bits(values, self.elem_bytes, "values")
        N.check(N.load().sg_vector_insert(self._h, _ptr(values), values.numel(), _stream(stream)), "vector::insert")

    def erase(self, n: int, stream=None) -> None:
        """erase(device_end() - n, device_end())."""
        N.check(N.load().sg_vector_erase(self._h, int(n), _stream(stream)), "vector::erase")

    def data(self) -> torch.Tensor:
        v = N.sg_vector_view()
        N.check(N.load().sg_vector_view_of(self._h, byref(v)), "vector::data")
        n = self.size()
        return _tensor_from_ptr(v.data, n, self.elem_bytes)


class deque:
    """stdgpu::deque<T> (T = 4 or 8 bytes): push_back / pop_front (src/stdgpu/deque.cuh)."""

    def __init__(self, handle: int, elem_bytes: int, capacity: int):
        self._h = c_void_p(handle)
        self.elem_bytes = elem_bytes
        self._capacity = capacity

    @classmethod
    def createDeviceObject(cls, capacity: int, elem_bytes: int = 8) -> "deque":
        h = c_void_p()
        N.check(N.load().sg_deque_create(elem_bytes, int(capacity), byref(h)), "deque::createDeviceObject")
        return cls(h.value, elem_bytes, capacity)

    @staticmethod
    def destroyDeviceObject(d: "deque") -> None:
        if d._h:
            N.check(N.load().sg_deque_destroy(d._h), "deque::destroyDeviceObject")
            d._h = c_void_p(0)

    def ops(self, is_push: torch.Tensor | None, values: torch.Tensor, *, stream=None):
        """One launch: element i push_back(values[i]) if is_push[i] else pop_front().  Returns (popped, ok)."""
        values = _as_bits(values, self.elem_bytes, "values")
        n = values.numel()
        popped = torch.zeros(n, dtype=_INT_DTYPE[self.elem_bytes], device=values.device)
        ok = torch.zeros(n, dtype=torch.uint8, device=values.device)
        N.check(N.load().sg_deque_ops(self._h, _ptr(is_push), _ptr(values), n, _ptr(popped), _ptr(ok),
                                      _stream(stream)), "deque::ops")
        return popped, ok

    def size(self, stream=None) -> int:
        out = c_int64()
        N.check(N.load().sg_deque_size(self._h, _stream(stream), byref(out)), "deque::size")
        return out.value

    def to_tensor(self, stream=None) -> torch.Tensor:
        out = torch.empty(max(self._capacity, 1), dtype=_INT_DTYPE[self.elem_bytes], device="cuda")
        n = c_int64()
        N.check(N.load().sg_deque_copy_out(self._h, _ptr(out), _stream(stream), byref(n)), "deque::copy_out")
        return out[: n.value]

    def clear(self, stream=None) -> None:
        N.check(N.load().sg_deque_clear(self._h, _stream(stream)), "deque::clear")

    def push_back(self, values: torch.Tensor, stream=None) -> torch.Tensor:
        values = _as_bits(values, self.elem_bytes, "values")
        return self.ops(None, values, stream=stream)[1]

    def pop_front(self, n: int, stream=None) -> tuple[torch.Tensor, torch.Tensor]:
        return self.ops(torch.zeros(n, dtype=torch.uint8, device="cuda"),
                        torch.zeros(n, dtype=_INT_DTYPE[self.elem_bytes], device="cuda"), stream=stream)

    def push_front(self, values: torch.Tensor, stream=None) -> torch.Tensor:
        """push_front() of each value in order (the last one ends at the front); returns ok flags."""
        values = _as_bits(values, self.elem_bytes, "values")
        ok = torch.zeros(values.numel(), dtype=torch.uint8, device=values.device)
        N.check(N.load().sg_deque_push_front(self._h, _ptr(values), values.numel(), _ptr(ok), _stream(stream)),
                "deque::push_front")
        return ok

    def pop_back(self, n: int, stream=None) -> tuple[torch.Tensor, torch.Tensor]:
        """pop_back() n times (the back element first); returns (values, ok)."""
        vals = torch.zeros(n, dtype=_INT_DTYPE[self.elem_bytes], device="cuda")
        ok = torch.zeros(n, dtype=torch.uint8, device="cuda")
        N.check(N.load().sg_deque_pop_back(self._h, int(n), _ptr(vals), _ptr(ok), _stream(stream)), "deque::pop_back")
        return vals, ok


class queue:
    """stdgpu::queue<T> (src/stdgpu/queue.cuh): push = deque::push_back, pop = deque::pop_front."""

    def __init__(self, d: deque):
        self.c = d

    @classmethod
    def createDeviceObject(cls, capacity: int, elem_bytes: int = 8) -> "queue":
        return cls(deque.createDeviceObject(capacity, elem_bytes))

    @staticmethod
    def destroyDeviceObject(q: "queue") -> None:
        deque.destroyDeviceObject(q.c)

    def push(self, values: torch.Tensor, stream=None) -> torch.Tensor:
        return self.c.push_back(values, stream)

    def pop(self, n: int, stream=None) -> tuple[torch.Tensor, torch.Tensor]:
        return self.c.pop_front(n, stream)

    def size(self, stream=None) -> int:
        return self.c.size(stream)

    def empty(self, stream=None) -> bool:
        return self.size(stream) == 0


class stack:
    """stdgpu::stack<T> (src/stdgpu/stack.cuh): push = deque::push_back, pop = deque::pop_back."""

    def __init__(self, d: deque):
        self.c = d

    @classmethod
    def createDeviceObject(cls, capacity: int, elem_bytes: int = 8) -> "stack":
        return cls(deque.createDeviceObject(capacity, elem_bytes))

    @staticmethod
    def destroyDeviceObject(s: "stack") -> None:
        deque.destroyDeviceObject(s.c)

    def push(self, values: torch.Tensor, stream=None) -> torch.Tensor:
        return self.c.push_back(values, stream)

    def pop(self, n: int, stream=None) -> tuple[torch.Tensor, torch.Tensor]:
        return self.c.pop_back(n, stream)

    def size(self, stream=None) -> int:
        return self.c.size(stream)

    def empty(self, stream=None) -> bool:
        return self.size(stream) == 0


def bitset_count(blocks: torch.Tensor, nbits: int, stream=None) -> int:
    """bitset<unsigned int>::count() over raw 32-bit blocks (src/stdgpu/impl/bitset_detail.cuh:388-404)."""
    blocks = _as_bits(blocks, 4, "blocks")
    if blocks.numel() * 32 < nbits:
        raise ValueError("blocks too short for nbits")
    out = c_int64()
    N.check(N.load().sg_bitset_count(_ptr(blocks), int(nbits), _stream(stream), byref(out)), "bitset::count")
    return out.value


def kernel_launch_count() -> int:
    return int(N.load().sg_kernel_launch_count())


class _DeviceArray:
    """Zero-copy description of a raw device buffer (CUDA array interface)."""

    def __init__(self, ptr: int, n: int, elem_bytes: int):
        self.__cuda_array_interface__ = {"shape": (n,), "typestr": "<i%d" % elem_bytes, "data": (ptr, False),
                                         "version": 3, "strides": None}


def _tensor_from_ptr(ptr: int, n: int, elem_bytes: int) -> torch.Tensor:
    """Copy n elements from a raw device pointer into a new tensor."""
    if n == 0:
        return torch.empty(0, dtype=_INT_DTYPE[elem_bytes], device="cuda")
    return torch.as_tensor(_DeviceArray(ptr, n, elem_bytes), device="cuda").clone()

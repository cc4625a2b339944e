"""The voxel-block map step, as the benchmark times it, and its element-by-element check.

Workload: stdgpu::unordered_map<uint64_t, uint32_t> of capacity 2 n; n unique voxel-block keys
(packed int3 surface voxels of 64 spheres, ``workloads.voxel_map``), values = insertion index.  One
step, on one stream, through the C ABI:

    sg_unordered_clear -> sg_unordered_insert(n value_type pairs, no flags)
      -> sg_unordered_find(n queries, 70 % hits) -> sg_unordered_erase(n / 4 keys, no flags)

At n = 2^27 the insert and erase calls take the partitioned path (scatter by home-group range, ordered
insert / erase, gated direct kernel).  ``VoxelStep.checked_step`` runs one step with a size read between
the calls and compares every result with values computed independently by torch sorting on the device:
the found flags against the generator's membership flags, every found value against the key's
insertion index, and the table's final contents against the keys minus the erased set with their
values.
"""

from __future__ import annotations

from ctypes import c_void_p

import numpy as np
import torch

from . import containers as C
from . import workloads as W
from ._native import load


class VoxelStep:
    def __init__(self, keys_log2: int, device: torch.device, hit_frac: float = 0.7, erase_frac: float = 0.25,
                 seed: int = 0, workload: W.VoxelWorkload | None = None):
        self.n = 1 << keys_log2
        self.capacity = 1 << (keys_log2 + 1)
        self.device = device
        self.w = workload if workload is not None else W.voxel_map(self.n, hit_frac=hit_frac,
                                                                    erase_frac=erase_frac, seed=seed)
        w = self.w
        self.n_q, self.n_e = len(w.queries), len(w.erase)
        # value_type array: pair<const uint64_t, uint32_t> = 16 bytes (key, value, 4 bytes padding)
        pairs_np = np.zeros((self.n, 2), np.uint64)
        pairs_np[:, 0] = w.keys
        pairs_np[:, 1] = w.values.astype(np.uint64)
        self.pairs_np = pairs_np.reshape(-1)
        to_dev = lambda a: torch.from_numpy(np.ascontiguousarray(a).view(np.int64)).to(device)
        self.pairs = to_dev(self.pairs_np)
        self.queries = to_dev(w.queries)
        self.erase = to_dev(w.erase)
        self.out_vals = torch.empty(self.n_q, dtype=torch.int32, device=device)
        self.out_found = torch.empty(self.n_q, dtype=torch.uint8, device=device)
        self.table = C.unordered_map.createDeviceObject(self.capacity, key="u64", mapped="u32")
        self.lib = load()
        self.h = self.table._h

    @property
    def ops_per_step(self) -> int:
        return self.n + self.n_q + self.n_e

    @staticmethod
    def _call(status: int, what: str) -> None:
        if status != 0:
            raise RuntimeError(f"{what} failed with status {status}")

    def clear(self, sp) -> None:
        self._call(self.lib.sg_unordered_clear(self.h, sp), "clear")

    def insert(self, sp) -> None:
        self._call(self.lib.sg_unordered_insert(self.h, c_void_p(self.pairs.data_ptr()), self.n, None, sp), "insert")

    def find(self, sp) -> None:
        self._call(self.lib.sg_unordered_find(self.h, c_void_p(self.queries.data_ptr()), self.n_q,
                                              c_void_p(self.out_vals.data_ptr()), c_void_p(self.out_found.data_ptr()),
                                              sp), "find")

    def erase_call(self, sp) -> None:
        self._call(self.lib.sg_unordered_erase(self.h, c_void_p(self.erase.data_ptr()), self.n_e, None, sp), "erase")

    def step(self, stream: torch.cuda.Stream, events=None) -> None:
        """clear, insert, find, erase on `stream`; events[0..4] (optional) are recorded around the calls."""
        sp = c_void_p(stream.cuda_stream)
        calls = (self.clear, self.insert, self.find, self.erase_call)
        for i, fn in enumerate(calls):
            if events is not None:
                events[i].record(stream)
            fn(sp)
        if events is not None:
            events[4].record(stream)

    def checked_step(self, stream: torch.cuda.Stream) -> dict:
        """One step with the table's size read after each call and every result compared with an
        independent torch computation; raises on the first difference.  Returns what it saw."""
        sp = c_void_p(stream.cuda_stream)
        dev = self.device
        seen = {}
        self.out_found.fill_(2)
        self.out_vals.fill_(-1)
        self.clear(sp)
        seen["size_after_clear"] = self.table.size(stream)
        l0 = C.kernel_launch_count()
        self.insert(sp)
        seen["insert_launches"] = C.kernel_launch_count() - l0
        seen["size_after_insert"] = self.table.size(stream)
        self.find(sp)
        l0 = C.kernel_launch_count()
        self.erase_call(sp)
        seen["erase_launches"] = C.kernel_launch_count() - l0
        seen["size_after_erase"] = self.table.size(stream)
        torch.cuda.synchronize(dev)

        def fail(msg):
            raise RuntimeError(f"voxel step wrong: {msg} ({seen})")

        if seen["size_after_clear"] != 0:
            fail("size after clear")
        if seen["size_after_insert"] != self.n:
            fail(f"size after insert {seen['size_after_insert']} != {self.n}")
        if seen["size_after_erase"] != self.n - self.n_e:
            fail(f"size after erase {seen['size_after_erase']} != {self.n - self.n_e}")

        keys = self.pairs.view(-1, 2)[:, 0]
        sorted_k, perm = torch.sort(keys)
        pos = torch.searchsorted(sorted_k, self.queries).clamp_(max=self.n - 1)
        hit = sorted_k[pos] == self.queries
        want_hit = torch.from_numpy(self.w.query_hit).to(dev)
        if not torch.equal(hit, want_hit):
            fail("the generator's membership flags disagree with the key set")
        found = self.out_found.bool()
        if not bool(((self.out_found == 0) | (self.out_found == 1)).all()):
            fail("find wrote a flag other than 0 / 1")
        if not torch.equal(found, hit):
            fail(f"found flags differ at {int((found != hit).sum())} queries")
        want_vals = perm[pos].to(torch.int32)  # values are the insertion index
        if not torch.equal(self.out_vals[hit], want_vals[hit]):
            fail(f"found values differ at {int((self.out_vals[hit] != want_vals[hit]).sum())} queries")

        # contents after the erase: the keys minus the erased ones, each with its insertion index
        epos = torch.searchsorted(sorted_k, self.erase)
        erased = torch.zeros(self.n, dtype=torch.bool, device=dev)
        erased[perm[epos]] = True
        if int(erased.sum()) != self.n_e:
            fail("erase keys are not distinct members")
        idx = torch.arange(self.n, dtype=torch.int64, device=dev)
        rem_k = keys[~erased]
        rem_v = idx[~erased].to(torch.int32)
        o = torch.argsort(rem_k)
        rem_k, rem_v = rem_k[o], rem_v[o]
        got_k, got_v = self.table.range_copy(stream)
        torch.cuda.synchronize(dev)
        if got_k.numel() != rem_k.numel():
            fail(f"range holds {got_k.numel()} elements, want {rem_k.numel()}")
        o = torch.argsort(got_k)
        if not torch.equal(got_k[o], rem_k):
            fail("final key set differs")
        if not torch.equal(got_v[o], rem_v):
            fail("final values differ")
        seen["checked_queries"] = self.n_q
        seen["checked_elements"] = int(rem_k.numel())
        return seen

    def close(self) -> None:
        C.unordered_base.destroyDeviceObject(self.table)

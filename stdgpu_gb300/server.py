"""Python mirror of the served request stream (include/stdgpu_gb300.h, sg_server_*).

The scheduler runs natively inside the library (stdgpu_gb300/csrc/server.cu); this class only submits
requests and keeps each request's device buffers alive until it completes.
"""

from __future__ import annotations

from ctypes import byref, c_double, c_int32, c_int64, c_void_p

import torch

from . import _native as N
from .containers import KINDS, _as_bits, _INT_DTYPE, _KEY_BYTES, _MAPPED_BYTES, _ptr

INSERT, FIND, ERASE = 0, 1, 2


class server:
    def __init__(self, key: str = "u64", mapped: str | None = "u64", budget_bytes: int = 120 << 30,
                 n_streams: int = 8, n_slots: int = 16):
        self.kind = KINDS[(key, mapped)]
        self.key_bytes = _KEY_BYTES[self.kind]
        self.mapped_bytes = _MAPPED_BYTES[self.kind]
        h = c_void_p()
        N.check(N.load().sg_server_create(self.kind, int(budget_bytes), n_streams, n_slots, byref(h)),
                "server::create")
        self._h = h
        self._live: dict[int, tuple] = {}

    def close(self) -> None:
        if self._h:
            N.check(N.load().sg_server_destroy(self._h), "server::destroy")
            self._h = c_void_p(0)
            self._live.clear()

    def admit(self, table: int, capacity: int) -> int:
        """createDeviceObject(capacity) under the budget; returns the status (SG_OK or SG_ERR_BUDGET)."""
        st = N.load().sg_server_admit_table(self._h, int(table), int(capacity))
        N.check(st, "server::admit", allow=(N.SG_ERR_BUDGET,))
        return st

    def drop(self, table: int) -> None:
        N.check(N.load().sg_server_drop_table(self._h, int(table)), "server::drop")

    def submit(self, table: int, op: int, keys: torch.Tensor, mapped: torch.Tensor | None = None,
               out_mapped: torch.Tensor | None = None, out_flags: torch.Tensor | None = None) -> int:
        keys = _as_bits(keys, self.key_bytes, "keys")
        if mapped is not None:
            mapped = _as_bits(mapped, self.mapped_bytes, "mapped")
        r = N.sg_request(int(table), int(op), keys.numel(), _ptr(keys).value, _ptr(mapped).value,
                         _ptr(out_mapped).value, _ptr(out_flags).value)
        t = c_int64()
        N.check(N.load().sg_server_submit(self._h, byref(r), byref(t)), "server::submit")
        self._live[t.value] = (keys, mapped, out_mapped, out_flags)
        return t.value

    def submit_many(self, items) -> list[int]:
        """items: (table, op, keys, mapped, out_mapped, out_flags) tuples, submitted in order in one call."""
        n = len(items)
        arr = (N.sg_request * n)()
        for k, (table, op, keys, mapped, out_mapped, out_flags) in enumerate(items):
            keys = _as_bits(keys, self.key_bytes, "keys")
            arr[k] = N.sg_request(int(table), int(op), keys.numel(), _ptr(keys).value, _ptr(mapped).value,
                                  _ptr(out_mapped).value, _ptr(out_flags).value)
        tickets = (c_int64 * n)()
        N.check(N.load().sg_server_submit_many(self._h, arr, n, tickets), "server::submit_many")
        out = list(tickets)
        for tk, it in zip(out, items):
            self._live[tk] = it
        return out

    def set_policy(self, direct_keys: int = 1 << 16, chunk_keys: int = 1 << 22, max_direct: int = 8,
                   direct_streams: int = 4) -> None:
        """Runs of at least direct_keys keys run as their own launches of at most chunk_keys keys on one of
        direct_streams low-priority streams, at most max_direct of them issued and not complete
        (sg_server_set_policy)."""
        N.check(N.load().sg_server_set_policy(self._h, int(direct_keys), int(chunk_keys), int(max_direct),
                                              int(direct_streams)), "server::set_policy")

    def set_grow_ahead(self, enabled: bool) -> None:
        """Growing ahead of idle tables more than half full (sg_server_set_grow_ahead; on by default)."""
        N.check(N.load().sg_server_set_grow_ahead(self._h, int(bool(enabled))), "server::set_grow_ahead")

    def pause(self, paused: bool = True) -> None:
        N.check(N.load().sg_server_set_paused(self._h, int(bool(paused))), "server::pause")

    def wait(self, ticket: int, timeout_ms: int = -1) -> int:
        st = c_int32()
        N.check(N.load().sg_server_wait(self._h, int(ticket), int(timeout_ms), byref(st)), "server::wait")
        self._live.pop(ticket, None)
        return st.value

    def drain(self, timeout_ms: int = -1) -> None:
        N.check(N.load().sg_server_drain(self._h, int(timeout_ms)), "server::drain")
        self._live.clear()

    def stats(self) -> dict:
        s = N.sg_server_stats()
        N.check(N.load().sg_server_get_stats(self._h, byref(s)), "server::stats")
        return {f: getattr(s, f) for f, _ in N.sg_server_stats._fields_}

    def latency_us(self, ticket: int) -> float:
        """Submission-to-completion latency of a completed request (sg_server_request_latency)."""
        x = c_double()
        N.check(N.load().sg_server_request_latency(self._h, int(ticket), byref(x)), "server::latency")
        return x.value

    def table_size(self, table: int) -> int:
        n = c_int64()
        N.check(N.load().sg_server_table_size(self._h, int(table), byref(n)), "server::table_size")
        return n.value

    def table_view(self, table: int) -> N.sg_unordered_view:
        v = N.sg_unordered_view()
        N.check(N.load().sg_server_table_view(self._h, int(table), byref(v)), "server::table_view")
        return v

    def new_outputs(self, n: int, device="cuda"):
        vals = torch.zeros(n, dtype=_INT_DTYPE[self.mapped_bytes], device=device) if self.mapped_bytes else None
        flags = torch.zeros(n, dtype=torch.uint8, device=device)
        return vals, flags

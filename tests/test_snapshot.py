"""Snapshot files: the loader rejects what is not a snapshot of a table the geometry allows, before it
allocates anything (no device needed for these cases)."""

import struct

import pytest

import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N


def header(kind=2, capacity=1 << 10, version=1, bucket_count=None, max_size=None, num_groups=None,
           bucket_heads_bytes=0, slot_heads_bytes=0):
    g = sg.geometry_for(2, capacity)
    b = g.bucket_count if bucket_count is None else bucket_count
    m = g.max_size if max_size is None else max_size
    ng = g.num_groups if num_groups is None else num_groups
    h = b"SGGB300T" + struct.pack("<IiII", version, kind, 0, g.slot_bytes)
    h += struct.pack("<qqqqqq", capacity, b, m, ng, 64, (ng + 1) * 128)
    if version >= 2:
        h += struct.pack("<qq", bucket_heads_bytes, slot_heads_bytes)
    return h + bytes(128 - len(h))


def load_status(path):
    from ctypes import byref, c_void_p
    h = c_void_p()
    st = sg.load().sg_unordered_load(str(path).encode(), None, byref(h))
    assert not h.value
    return st


@pytest.mark.parametrize("content", [b"", b"not a snapshot", b"SGGB300T" + bytes(200)])
def test_load_rejects_garbage(tmp_path, content):
    f = tmp_path / "bad.sgt"
    f.write_bytes(content)
    assert load_status(f) == N.SG_ERR_BAD_ARG


@pytest.mark.parametrize("tweak", [dict(version=3), dict(version=0), dict(bucket_count=999), dict(max_size=5),
                                   dict(num_groups=1), dict(kind=9),
                                   # version 2: the accounting's bit arrays must match the geometry
                                   dict(version=2, bucket_heads_bytes=4, slot_heads_bytes=4),
                                   dict(version=2, bucket_heads_bytes=1 << 40, slot_heads_bytes=8)])
def test_load_rejects_inconsistent_header(tmp_path, tweak):
    f = tmp_path / "bad.sgt"
    f.write_bytes(header(**tweak))
    assert load_status(f) == N.SG_ERR_BAD_ARG


def test_load_missing_file(tmp_path):
    assert load_status(tmp_path / "absent.sgt") == N.SG_ERR_BAD_ARG

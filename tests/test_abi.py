"""The C-ABI library builds, loads and exports every entry point that include/stdgpu_gb300.h declares.

CPU only: no compute call is made (there is no device here).
"""

import re
from pathlib import Path

import stdgpu_gb300
from stdgpu_gb300 import _native as N

HEADER = Path(__file__).resolve().parents[1] / "include" / "stdgpu_gb300.h"


def declared_symbols():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"^SG_API\s+[\w\s\*]+?\b(sg_\w+)\s*\(", text, flags=re.M)))


def test_header_declarations_parsed():
    syms = declared_symbols()
    assert "sg_unordered_insert" in syms and "sg_bitset_count" in syms
    assert len(syms) >= 30


def test_library_exports_every_declared_symbol():
    lib = stdgpu_gb300.load()
    missing = [s for s in declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing


def test_binding_table_covers_header():
    assert set(declared_symbols()) == set(N.SIGNATURES)


def test_status_strings_without_device():
    lib = stdgpu_gb300.load()
    assert lib.sg_status_string(N.SG_OK) == b"ok"
    assert b"full" in lib.sg_status_string(N.SG_ERR_FULL)


def test_geometry_query_without_device():
    # host-only entry point: createDeviceObject geometry for the benchmark capacities
    g = stdgpu_gb300.geometry_for(N.MAP_U64_U32, 1 << 28)
    assert (g.bucket_count, g.max_size) == (268435456, 438119028)
    assert g.slot_bytes == 16 and g.slots_per_group == 8
    assert g.num_groups * g.slots_per_group >= g.max_size
    g1 = stdgpu_gb300.geometry_for(N.SET_U32, 1)
    assert (g1.bucket_count, g1.max_size, g1.num_groups) == (1, 2, 1)


def test_bad_arguments_rejected_without_device():
    lib = stdgpu_gb300.load()
    g = N.sg_geometry()
    import ctypes
    assert lib.sg_unordered_geometry_for(99, 10, ctypes.byref(g)) == N.SG_ERR_BAD_ARG
    assert lib.sg_unordered_geometry_for(N.SET_U32, 0, ctypes.byref(g)) == N.SG_ERR_BAD_ARG
    # max_size must fit the reference's 32-bit index_t
    assert lib.sg_unordered_geometry_for(N.SET_U32, 1 << 31, ctypes.byref(g)) == N.SG_ERR_BAD_ARG
    assert lib.sg_unordered_insert(None, None, 0, None, None) == N.SG_ERR_BAD_ARG
    assert lib.sg_bitset_count(None, 5, None, None) == N.SG_ERR_BAD_ARG

"""The device allocator hook (sg_set_device_allocator): CPU part -- installing and removing a pair while
nothing is allocated, rejecting half a pair."""

import ctypes

import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N

ALLOC = ctypes.CFUNCTYPE(ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p)
FREE = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p)


def test_install_and_remove_without_live_storage():
    lib = sg.load()
    assert sg.live_device_allocations() == 0
    a = ALLOC(lambda n, ctx: None)
    f = FREE(lambda p, ctx: None)
    pa, pf = ctypes.cast(a, ctypes.c_void_p), ctypes.cast(f, ctypes.c_void_p)
    assert lib.sg_set_device_allocator(pa, None, None) == N.SG_ERR_BAD_ARG
    assert lib.sg_set_device_allocator(None, pf, None) == N.SG_ERR_BAD_ARG
    assert lib.sg_set_device_allocator(pa, pf, None) == N.SG_OK
    assert lib.sg_set_device_allocator(None, None, None) == N.SG_OK

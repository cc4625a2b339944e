"""sg_measure_random_reads: argument checks on the CPU, a small measurement on the GPU."""

from ctypes import byref, c_double

import pytest

import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N


def test_random_reads_rejects_bad_arguments():
    lib = sg.load()
    r = c_double(0.0)
    assert lib.sg_measure_random_reads(1 << 19, 1000, 128, None, byref(r)) == N.SG_ERR_BAD_ARG  # buffer < 1 MiB
    assert lib.sg_measure_random_reads(1 << 24, 0, 128, None, byref(r)) == N.SG_ERR_BAD_ARG
    assert lib.sg_measure_random_reads(1 << 24, 1000, 48, None, byref(r)) == N.SG_ERR_BAD_ARG
    assert lib.sg_measure_random_reads(1 << 24, 1000, 128, None, None) == N.SG_ERR_BAD_ARG


@pytest.mark.gpu
@pytest.mark.parametrize("unit", [32, 64, 128])
def test_random_reads_measures_a_rate(unit):
    import torch
    lib = sg.load()
    r = c_double(0.0)
    s = torch.cuda.current_stream()
    from ctypes import c_void_p
    assert lib.sg_measure_random_reads(1 << 30, 1 << 22, unit, c_void_p(s.cuda_stream), byref(r)) == 0
    # far above any host-side rate, far below one read per SM clock on every SM of the GPU
    assert 1e9 < r.value < 152 * 2.1e9 * 4

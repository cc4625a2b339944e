"""Device calls and custom key types through the C++ API (stdgpu_gb300/device_bench.cu), at a size the GPU
suite runs in seconds: device insert / find / erase of a native map (every found value is its inserting
thread's index, sizes after each launch), and voxel-coordinate sets of 3 x int16 (word-keyed) and
3 x int32 (wide) keys with the caller's spatial hash (bulk insert, device contains of every stored key and
of keys outside the cube, device insert of new keys, bulk erase; sizes and valid())."""

import pytest


def test_device_bench_program_compiles_for_sm103a():
    """CPU part: the program builds against the library for sm_103a (no device needed)."""
    import stdgpu_gb300
    from stdgpu_gb300 import device_bench
    stdgpu_gb300.load()
    assert device_bench.build().exists()


@pytest.mark.gpu
@pytest.mark.parametrize("keys_log2", [12, 18])
def test_device_calls_and_custom_keys(keys_log2):
    from stdgpu_gb300 import device_bench
    r = device_bench.run(keys_log2=keys_log2, timeout=300)
    assert r["returncode"] == 0, r
    assert len(r["parts"]) == 3, r
    for p in r["parts"]:
        assert p["checks_pass"], p

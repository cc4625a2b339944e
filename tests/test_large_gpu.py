"""The large mixed workload (map at 0.5 / 0.75 / 0.9 load with Zipf batches, vector, deque, bitset) at a
reduced scale; each part checks its own result with size-independent properties."""

import pytest

from stdgpu_gb300 import large_bench

pytestmark = pytest.mark.gpu


def test_large_workload_reduced_scale_checks_pass():
    r = large_bench.run(full=False)
    for m in r["map"][:-1]:
        assert m["checks_pass"], m
        assert m["size_after_prefill"] == m["expected_size"]
    assert r["map"][-1]["valid"]
    assert r["vector"]["checks_pass"], r["vector"]
    assert r["deque"]["checks_pass"], r["deque"]
    assert r["bitset"]["checks_pass"], r["bitset"]

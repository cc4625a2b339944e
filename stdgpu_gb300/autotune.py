"""Autotuner of the batched many-table kernels' launch shape, run on a GB300.

Sweeps threads per block x resident blocks per SM x tiles taken per warp step on the many-small-tables
workload (stdgpu_gb300/batch_bench.py: clear + insert + contains of 4096 lognormal-sized sets), times
each shape with CUDA events (best of 3 runs of 3 steps) and records every result and the fastest shape
in stdgpu_gb300/tuning/batch.json, which table_batch.createDeviceObjects applies.  The probe-group width
(128 bytes, one request per group) and the table geometry (the reference's bucket / excess counts)
are fixed: the first by measurement of random-line reads on this GPU, the second for parity of
max_size() and bucket_count().

    python -m stdgpu_gb300.autotune
"""

from __future__ import annotations

import json
import time
from pathlib import Path

import torch

from . import batch_bench as BB
from . import containers as C

OUT = Path(__file__).resolve().parent / "tuning" / "batch.json"
SHAPES = [(t, b, k) for t in (128, 256, 512) for b in (0, 1, 2, 4) for k in (1, 2, 4, 8)]


def main() -> dict:
    counts, caps, keys, queries, offsets = BB.make_workload()
    d_keys, d_q, d_off = BB.to_dev(keys), BB.to_dev(queries), BB.to_dev(offsets)
    out = torch.zeros(len(queries), dtype=torch.uint8, device="cuda")
    batch = C.table_batch.createDeviceObjects(caps, key="u64", tuning={"threads_per_block": 256,
                                                                      "blocks_per_sm": 0, "tiles_per_step": 1})
    results = []
    for threads, bpsm, tiles in SHAPES:
        batch.configure(threads, bpsm, tiles)
        ms = min(BB.time_batched(batch, d_keys, d_q, d_off, out, steps=3, warmup=1) for _ in range(3))
        results.append({"threads_per_block": threads, "blocks_per_sm": bpsm, "tiles_per_step": tiles,
                        "ms_per_step": ms})
    C.table_batch.destroyDeviceObjects(batch)
    best = min(results, key=lambda r: r["ms_per_step"])
    record = {
        "workload": "4096 unordered_set<uint64_t>, lognormal counts (median 2048, sigma 1.5), clear+insert+contains",
        "gpu": torch.cuda.get_device_name(0),
        "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
        "best": {k: best[k] for k in ("threads_per_block", "blocks_per_sm", "tiles_per_step")},
        "best_ms_per_step": best["ms_per_step"],
        "results": results,
    }
    OUT.parent.mkdir(exist_ok=True)
    OUT.write_text(json.dumps(record, indent=1) + "\n")
    return record


if __name__ == "__main__":
    r = main()
    print(json.dumps({"best": r["best"], "best_ms_per_step": r["best_ms_per_step"]}))

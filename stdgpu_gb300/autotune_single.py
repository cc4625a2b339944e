"""Autotuner of the single-table kernels' launch shapes, run on a GB300.

The shapes are compile-time constants of stdgpu_gb300/csrc/unordered.cu and table_core.cuh:

* SG_STAGE_ITERS        -- keys per warp per chunk of the staged ordered insert, in 32s (chunk = 256 x it)
* SG_ERASE_ORDERED_ITERS -- the same for the ordered erase (chunk = 256 x it keys)
* SG_PART_REGION_MB     -- bytes of slots per partition of the partitioned bulk calls
* SG_BULK_MIN_BLOCKS    -- resident blocks per SM the probe kernels are compiled for (registers per thread)

Each candidate is built into its own library (build.build with explicit flags), and the voxel-map step
(clear, insert of value_type pairs, find at 70 % hits, erase 25 %; stdgpu_gb300/voxel_step.py) is timed
with it in a fresh process (STDGPU_GB300_LIB) after the step has been checked element by element.  The
sweep is coordinate descent from the current shapes: one knob at a time, keeping the fastest.  Every
result and the best shapes go to stdgpu_gb300/tuning/single_table.json, which build.py applies.  The
probe-group width (128 bytes) and the table geometry are fixed (random-line reads on this GPU; parity of
max_size() and bucket_count()).

    python -m stdgpu_gb300.autotune_single [--keys-log2 27]
"""

from __future__ import annotations

import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

from . import build as B

KNOBS = {
    "SG_STAGE_ITERS": [2, 4],
    "SG_ERASE_ORDERED_ITERS": [1, 2, 4],
    "SG_PART_REGION_MB": [32, 64, 128],
    "SG_BULK_MIN_BLOCKS": [3, 4],
}
START = {"SG_STAGE_ITERS": 4, "SG_ERASE_ORDERED_ITERS": 2, "SG_PART_REGION_MB": 64, "SG_BULK_MIN_BLOCKS": 4}


def time_step(keys_log2: int, steps: int = 10) -> dict:
    """Phase times (median ms) of the voxel step with the library this process loads, after one checked step."""
    import numpy as np
    import torch

    from . import workloads as W
    from .voxel_step import VoxelStep

    cache = Path(tempfile.gettempdir()) / f"sg_voxel_{keys_log2}.npz"
    if cache.exists():
        z = np.load(cache)
        w = W.VoxelWorkload(z["keys"], z["values"], z["queries"], z["query_hit"], z["erase"])
    else:
        w = W.voxel_map(1 << keys_log2, hit_frac=0.7, erase_frac=0.25, seed=0)
        np.savez(cache, keys=w.keys, values=w.values, queries=w.queries, query_hit=w.query_hit, erase=w.erase)
    vs = VoxelStep(keys_log2, torch.device("cuda", 0), workload=w)
    st = torch.cuda.current_stream()
    vs.checked_step(st)
    for _ in range(3):
        vs.step(st)
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(steps)]
    torch.cuda.synchronize()
    for e in evs:
        vs.step(st, e)
    torch.cuda.synchronize()
    out = {n: statistics.median(e[i].elapsed_time(e[i + 1]) for e in evs)
           for i, n in enumerate(["clear", "insert", "find", "erase"])}
    out["step"] = statistics.median(e[0].elapsed_time(e[4]) for e in evs)
    vs.close()
    return out


def measure(shape: dict, keys_log2: int, work: Path) -> dict:
    tag = "_".join(f"{k[3:].lower()}{v}" for k, v in sorted(shape.items()))
    lib = work / f"lib_{tag}.so"
    if not lib.exists():
        B.build(flags=[f"-D{k}={v}" for k, v in sorted(shape.items())], out_lib=lib)
    env = dict(os.environ, STDGPU_GB300_LIB=str(lib))
    r = subprocess.run([sys.executable, "-m", "stdgpu_gb300.autotune_single", "--time", "--keys-log2", str(keys_log2)],
                       capture_output=True, text=True, env=env, cwd=B.ROOT)
    if r.returncode != 0:
        return {"shape": shape, "error": r.stderr[-500:]}
    return {"shape": shape, **json.loads(r.stdout.strip().splitlines()[-1])}


def main(keys_log2: int = 27) -> dict:
    work = Path(tempfile.mkdtemp(prefix="sg_tune_"))
    results = []
    best_shape = dict(START)
    best = measure(best_shape, keys_log2, work)
    results.append(best)
    for knob, values in KNOBS.items():
        for v in values:
            if v == best_shape[knob]:
                continue
            cand = dict(best_shape, **{knob: v})
            r = measure(cand, keys_log2, work)
            results.append(r)
            if "step" in r and r["step"] < best["step"]:
                best, best_shape = r, cand
    record = {
        "workload": f"voxel-map step, 2^{keys_log2} keys, capacity 2^{keys_log2 + 1}: clear + insert + find + erase",
        "when": time.strftime("%Y-%m-%dT%H:%M:%SZ", time.gmtime()),
        "best": best_shape,
        "best_step_ms": best["step"],
        "results": results,
    }
    B.TUNING.parent.mkdir(exist_ok=True)
    B.TUNING.write_text(json.dumps(record, indent=1) + "\n")
    return record


if __name__ == "__main__":
    import argparse

    ap = argparse.ArgumentParser()
    ap.add_argument("--keys-log2", type=int, default=27)
    ap.add_argument("--time", action="store_true", help="time the step with the loaded library (one candidate)")
    a = ap.parse_args()
    if a.time:
        print(json.dumps(time_step(a.keys_log2)))
    else:
        rec = main(a.keys_log2)
        print(json.dumps({"best": rec["best"], "best_step_ms": rec["best_step_ms"]}))

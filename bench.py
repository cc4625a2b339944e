"""Benchmark of the hashed-container hot path on the voxel-block map workload.

Workload (one GPU): stdgpu::unordered_map<uint64_t, uint32_t> with capacity 2^28;
2^27 unique voxel-block keys (packed int3, 21 bits per axis, the surface voxels
of a union of 64 random spheres), values = insertion index.  One step is one
pass of the hot path on device-resident inputs:

    clear -> insert(2^27 value_type pairs) -> find(2^27 keys, 70% hits) -> erase(2^25 keys)

value = (inserts + finds + erases) / step time, in Mops/s, with CUDA events on
the stream the kernels run on.  Inputs (2 GiB of pairs, 1 GiB of queries) are
larger than L2, so no flush is needed between steps.

e2e: the same step through the C ABI's host-buffer entry points (sg_unordered_*_host):
every step copies its inputs host->device from pinned memory and the find results
device->host, in chunks overlapped with the kernels; the host inputs are static, so the
stager is told so (sg_stager_set_inputs_ready) and a call's uploads start while the previous
call's kernels run.  ordered_uploads: the same with uploads in stream order (the stager's
default).  serial_copies: whole-array copies before and after the device-pointer calls.

--impl reference: the reference's own CPU implementation (stdgpu 1.3.0,
OpenMP backend, built under oracle/_ref) on a bounded sample of the same
workload with all host threads; falls back to the oracle restatement when the
reference library is not available.

Multi-GPU (torchrun, N > 1): the path is not partitioned here; each rank runs
an independent replica of the workload ("replicas only"), and value sums the
ranks' operations over the slowest rank's time.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "insert/find Mops/s & HBM-roofline %"
UNIT = "Mops/s"
CAPACITY_LOG2 = 28
KEYS_LOG2 = 27
HIT_FRAC = 0.7
ERASE_FRAC = 0.25

# Algorithmic bytes per operation (lower bound; one 128-byte group line per op):
#   insert: 16 B value_type pair in + 128 B home group + one 32 B sector written back (key and value share it)
#   find:   8 B key in + 4 B value + 1 B flag out + 128 B home group (the value sits in the same line)
#   erase:  8 B key in + 128 B home group + one 32 B sector written back (the erased marker)
BYTES_PER_OP = {"insert": 16 + 128 + 32, "find": 8 + 5 + 128, "erase": 8 + 128 + 32}
NOMINAL_HBM_GBS = 7900.0  # HBM3e nominal, reported beside the measured copy peak
# the native arm's cpu_baseline: one host thread on 2^23 keys of the workload (capacity 2^24; the
# reference's arrays, about 0.3 GB, are larger than the host's caches)
CPU_BASELINE_KEYS_LOG2 = 23


def parse_args(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", choices=["native", "reference"], default="native")
    p.add_argument("--keys-log2", type=int, default=KEYS_LOG2, help="2^k keys (default: the full workload)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-other-configs", action="store_true",
                   help="skip the small / batched / served configurations that follow the voxel step")
    p.add_argument("--workload", choices=["voxel", "batched", "serve", "large", "small", "device"], default="voxel",
                   help="voxel: the headline map workload; batched: 4096 small sets, batched vs plain calls; "
                        "serve: request stream over 256 resident maps, continuous batching vs serial calls; "
                        "large: capacity-2^30 map at 0.5/0.75/0.9 load plus vector / deque / bitset; "
                        "small: an L2-resident 2^20-key set, eager and as one CUDA graph")
    p.add_argument("--requests", type=int, default=600, help="serve workload: number of requests")
    p.add_argument("--e2e-chunk-log2", type=int, default=22, help="e2e: elements per staged chunk, log2")
    p.add_argument("--e2e-buffers", type=int, default=4, help="e2e: staging buffers in the ring")
    p.add_argument("--ref-keys-log2", type=int, default=20,
                   help="reference arm, voxel workload: keys per timed sample step, log2")
    p.add_argument("--ref-full", action="store_true",
                   help="reference arm: time the voxel workload at --keys-log2 itself instead of a sample")
    p.add_argument("--ref-threads", type=int, default=0, help="reference arm: host threads (default: all)")
    return p.parse_args(argv)


def parse():
    return parse_args()


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def slowest_rank_ms(ms: float, ws: int, device) -> float:
    """The largest per-step time over all ranks (every rank runs its own replica of the workload)."""
    if ws <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replicas_value(ops_per_step: int, ms: float, ws: int, device) -> tuple[float, float]:
    """(whole-job Mops/s, slowest rank's ms per step): all ranks' operations over the slowest rank's time."""
    worst = slowest_rank_ms(ms, ws, device)
    return ops_per_step * ws / (worst * 1e-3) / 1e6, worst


def link_bandwidth(host, device_buf, stream, device, reps: int = 3) -> dict:
    """Pinned host<->device copy bandwidth of this GPU's host link (GB/s), measured on the same box as the e2e
    step: the best of `reps` whole-buffer copies each way, CUDA events on the copying stream."""
    import torch
    nbytes = host.numel() * host.element_size()
    out = {}
    for name, dst, src in (("h2d_gbs", device_buf, host), ("d2h_gbs", host, device_buf)):
        best = None
        for _ in range(reps):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize(device)
            a.record(stream)
            dst.copy_(src, non_blocking=True)
            b.record(stream)
            torch.cuda.synchronize(device)
            ms = a.elapsed_time(b)
            best = ms if best is None else min(best, ms)
        out[name] = nbytes / (best * 1e-3) / 1e9
    return out


# ------------------------------------------------------------------ clocks

class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, max clock, throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        busy = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ CPU side

def cpu_sample_run(threads: int, keys_log2: int = 20, reps: int = 1):
    """Reference (or oracle restatement) on 2^keys_log2 keys of the voxel workload at the benchmark's load
    (capacity 2^(keys_log2+1)): returns (Mops/s, kind, threads used, sample text, phase seconds, step seconds)."""
    import oracle as O
    from stdgpu_gb300 import workloads as W

    n = 1 << keys_log2
    w = W.voxel_map(n, hit_frac=HIT_FRAC, erase_frac=ERASE_FRAC, seed=0)
    kind = "reference" if O.ref_available() else "port"
    if kind == "reference":
        O.ref_set_threads(threads)
        make = lambda: O.RefTable(O.MAP_U64_U32, 2 * n)
    else:
        threads = 1
        make = lambda: O.PortTable(O.MAP_U64_U32, 2 * n)
    best = None
    for _ in range(reps):
        t = make()
        t0 = time.perf_counter()
        t.insert(w.keys, w.values)
        t1 = time.perf_counter()
        t.find(w.queries)
        t2 = time.perf_counter()
        t.erase(w.erase)
        t3 = time.perf_counter()
        size = t.size()
        t.close()
        if size != n - len(w.erase):
            raise RuntimeError(f"{kind} size {size} after the sample step, want {n - len(w.erase)}")
        ops = len(w.keys) + len(w.queries) + len(w.erase)
        mops = ops / (t3 - t0) / 1e6
        if best is None or mops > best[0]:
            best = (mops, {"insert_s": t1 - t0, "find_s": t2 - t1, "erase_s": t3 - t2}, t3 - t0)
    sample = (f"2^{keys_log2} voxel keys into capacity 2^{keys_log2 + 1} (same 0.5 load), 2^{keys_log2} finds "
              f"(70% hits), {len(w.erase)} erases; insert+find+erase wall time, best of {reps}")
    return best[0], kind, threads, sample, best[1], best[2]


def std_map_sample(keys_log2: int = 21) -> dict:
    """Sanity line beside the reference: std::unordered_map<uint64_t, uint32_t> in one host thread on the same
    sample of the workload (insert, find 70 % hits, erase 25 %)."""
    import oracle as O
    from stdgpu_gb300 import workloads as W

    n = 1 << keys_log2
    w = W.voxel_map(n, hit_frac=HIT_FRAC, erase_frac=ERASE_FRAC, seed=0)
    secs, hits, _, size = O.ref_std_unordered_map(w.keys, w.values, w.queries, w.erase)
    ops = len(w.keys) + len(w.queries) + len(w.erase)
    return {"value": ops / secs / 1e6, "unit": UNIT, "cores": 1, "kind": "std::unordered_map",
            "sample": f"2^{keys_log2} voxel keys, 2^{keys_log2} finds ({hits} hits), {len(w.erase)} erases; "
                      f"final size {size}"}


def std_map_line(keys_log2: int) -> dict:
    try:
        return std_map_sample(keys_log2)
    except Exception as ex:  # the sanity line never costs the benchmark its result
        return {"unavailable": str(ex)[:200]}


def small_cpu_run(threads: int, reps: int = 1):
    """The small configuration at its full size on the host: unordered_set<uint32_t> capacity 2^21, 2^20
    uniform keys, 2^20 contains (50 % hits), erase of half the keys; (Mops/s, kind, threads, phase s, step s)."""
    import oracle as O
    from stdgpu_gb300 import small_bench

    keys, queries, erase = small_bench.make_inputs()
    kind = "reference" if O.ref_available() else "port"
    if kind == "reference":
        O.ref_set_threads(threads)
        make = lambda: O.RefTable(O.SET_U32, 1 << 21)
    else:
        threads = 1
        make = lambda: O.PortTable(O.SET_U32, 1 << 21)
    best = None
    for _ in range(reps):
        t = make()
        t0 = time.perf_counter()
        t.insert(keys)
        t1 = time.perf_counter()
        t.contains(queries)
        t2 = time.perf_counter()
        t.erase(erase)
        t3 = time.perf_counter()
        t.close()
        ops = len(keys) + len(queries) + len(erase)
        mops = ops / (t3 - t0) / 1e6
        if best is None or mops > best[0]:
            best = (mops, {"insert_s": t1 - t0, "contains_s": t2 - t1, "erase_s": t3 - t2}, t3 - t0)
    return best[0], kind, threads, best[1], best[2]


def reference_arm(args):
    """The reference's own CPU implementation (oracle/_ref, OpenMP backend) on the host cores.  Each step
    is the sample that the config names -- for the voxel workload 2^ref_keys_log2 keys at the benchmark's
    0.5 load (the 2^27-key workload itself takes minutes per step on the host), for the small workload the
    full configuration -- and ms_per_step is that step's measured wall time."""
    ws, rank, _ = dist_info()
    if rank != 0:
        return
    threads = args.ref_threads or os.cpu_count() or 1
    vals, step_s = [], []
    detail = None
    kind = sample = None
    if args.workload == "small":
        for i in range(args.warmup + args.steps):
            mops, kind, used, detail, secs = small_cpu_run(threads)
            if i >= args.warmup:
                vals.append(mops)
                step_s.append(secs)
        sample = "the full small configuration (2^20 keys, capacity 2^21): insert+contains+erase wall time"
        config = {"workload": "unordered_set<uint32_t>, capacity 2^21, 2^20 uniform keys; insert + contains "
                              "(50% hits) + erase half, per step", "capacity": 1 << 21, "keys": 1 << 20,
                  "finds": 1 << 20, "erases": 1 << 19}
        std_line = None
    else:
        k = args.keys_log2 if args.ref_full else args.ref_keys_log2
        for i in range(args.warmup + args.steps):
            mops, kind, used, sample, detail, secs = cpu_sample_run(threads, keys_log2=k, reps=1)
            if i >= args.warmup:
                vals.append(mops)
                step_s.append(secs)
        n = 1 << k
        config = {"workload": f"voxel-block unordered_map<uint64_t,uint32_t>, capacity 2^{k + 1}, 2^{k} keys; "
                              f"insert+find(70% hits)+erase(25%) per step",
                  "capacity": 2 * n, "keys": n, "finds": n, "erases": n // 4,
                  "native_arm_workload": f"the same generator at 2^{args.keys_log2} keys, capacity "
                                         f"2^{args.keys_log2 + 1}" + (" (this run)" if args.ref_full else
                                                                      " (this run times a sample of it)")}
        std_line = std_map_line(k) if k <= 24 else None
    value = statistics.median(vals)
    config.update({"parallelism": f"host threads ({used})", "l2": "not applicable (host)", "sampled": sample})
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.median(step_s) * 1e3,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u64" if args.workload != "small" else "u32", "data": "synthetic",
        "config": config,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": used, "kind": kind, "sample": sample,
                         "std_unordered_map": std_line},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "phases_s": detail,
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------ GPU side

def native_arm(args):
    import torch
    import stdgpu_gb300 as sg

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from stdgpu_gb300.voxel_step import VoxelStep

    vs = VoxelStep(args.keys_log2, dev, hit_frac=HIT_FRAC, erase_frac=ERASE_FRAC, seed=0)
    w = vs.w
    n, cap, n_q, n_e = vs.n, vs.capacity, vs.n_q, vs.n_e
    pairs_np = vs.pairs_np
    pairs, queries, erase = vs.pairs, vs.queries, vs.erase
    out_vals, out_found = vs.out_vals, vs.out_found
    table, lib, h = vs.table, vs.lib, vs.h
    from ctypes import c_void_p
    stream = torch.cuda.current_stream(dev)
    sp = c_void_p(stream.cuda_stream)

    def call(status, what):
        if status != 0:
            raise RuntimeError(f"{what} failed with status {status}")

    def step(ev=None):
        vs.step(stream, ev)

    # the random-read ceiling of this GPU's memory, on a buffer the size of the table (untimed, before the run)
    from ctypes import byref, c_double
    table_bytes = int(table.geometry().storage_bytes)
    rate = c_double(0.0)
    ceiling = None
    if lib.sg_measure_random_reads(table_bytes, n, 128, sp, byref(rate)) == 0 and rate.value > 0:
        ceiling = {"reads_per_s": rate.value, "unit_bytes": 128, "buffer_bytes": table_bytes,
                   "note": "random 128-byte reads per second of this GPU's memory (sg_measure_random_reads); "
                           "32- and 64-byte reads complete at the same rate, so a probe kernel that reads one "
                           "group line per key is bound by this count, not by bytes"}

    # correctness guard on the timed configuration (one untimed pass): sizes after every call, every found
    # flag and value, and the final contents compared element by element with an independent computation
    guard = vs.checked_step(stream)
    checked_found = out_found.cpu().numpy().astype(bool)
    checked_vals = out_vals.cpu()

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize(dev)
    if ws > 1:
        torch.distributed.barrier()

    sampler = ClockSampler(local)
    sampler.start()
    time.sleep(0.3)
    launches0 = sg.kernel_launch_count()
    evs = [[torch.cuda.Event(enable_timing=True) for _ in range(5)] for _ in range(args.steps)]
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize(dev)
    t_start.record(stream)
    for k in range(args.steps):
        step(evs[k])
    t_end.record(stream)
    torch.cuda.synchronize(dev)
    launches = sg.kernel_launch_count() - launches0
    clocks = sampler.stop()
    total_ms = t_start.elapsed_time(t_end)
    phase_ms = {name: [evs[k][i].elapsed_time(evs[k][i + 1]) for k in range(args.steps)]
                for i, name in enumerate(["clear", "insert", "find", "erase"])}
    ops_per_step = n + n_q + n_e
    value, ms_per_step = replicas_value(ops_per_step, total_ms / args.steps, ws, dev)

    # ---------------- e2e: host buffers through the C ABI, copies inside the timed region
    e2e = None
    if not args.no_e2e:
        pairs_h = torch.from_numpy(pairs_np.reshape(-1).view(np.int64)).pin_memory()
        queries_h = torch.from_numpy(w.queries.view(np.int64)).pin_memory()
        erase_h = torch.from_numpy(w.erase.view(np.int64)).pin_memory()
        vals_h = torch.empty(n_q, dtype=torch.int32).pin_memory()
        found_h = torch.empty(n_q, dtype=torch.uint8).pin_memory()

        stager = sg.stager(1 << args.e2e_chunk_log2, args.e2e_buffers)
        hp = lambda t: c_void_p(t.data_ptr())

        e2e_phase_ms = {"clear": [], "insert_host": [], "find_host": [], "erase_host": []}

        e2e_host_ms = {}

        def e2e_step(ev=None):
            # the host-buffer entry points: chunked copies in, kernels, results out, overlapped; with events,
            # the host time of each call is kept too (a call blocks the host while its staging buffers cycle)
            calls = (("clear", lambda: lib.sg_unordered_clear(h, sp)),
                     ("insert_host", lambda: lib.sg_unordered_insert_host(h, stager._h, hp(pairs_h), n, None, sp)),
                     ("find_host", lambda: lib.sg_unordered_find_host(h, stager._h, hp(queries_h), n_q, hp(vals_h),
                                                                      hp(found_h), sp)),
                     ("erase_host", lambda: lib.sg_unordered_erase_host(h, stager._h, hp(erase_h), n_e, None, sp)))
            if ev is not None:
                ev[0].record(stream)
            for k, (name, fn) in enumerate(calls):
                t0 = time.perf_counter()
                call(fn(), name)
                if ev is not None:
                    e2e_host_ms[name] = (time.perf_counter() - t0) * 1e3
                    ev[k + 1].record(stream)

        def e2e_serial_step():
            # the same step as separate whole-array copies around the device-pointer calls
            pairs.copy_(pairs_h, non_blocking=True)
            queries.copy_(queries_h, non_blocking=True)
            erase.copy_(erase_h, non_blocking=True)
            step()
            vals_h.copy_(out_vals, non_blocking=True)
            found_h.copy_(out_found, non_blocking=True)

        def time_steps(fn):
            for _ in range(args.warmup):
                fn()
            torch.cuda.synchronize(dev)
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            for _ in range(args.steps):
                fn()
            b.record(stream)
            torch.cuda.synchronize(dev)
            got = found_h.numpy().astype(bool)
            gm = torch.from_numpy(got)
            if (not np.array_equal(got, checked_found) or not torch.equal(vals_h[gm], checked_vals[gm])
                    or table.size() != n - n_e):
                raise RuntimeError("e2e results differ from the checked device-resident step")
            found_h.zero_()
            return a.elapsed_time(b) / args.steps

        # uploads in stream order (the stager's default), then with the inputs declared ready: the host
        # buffers are static here, so the uploads of a call may start while the previous call's kernels run
        ordered_ms = slowest_rank_ms(time_steps(e2e_step), ws, dev)
        stager.set_inputs_ready(True)
        e2e_ms = slowest_rank_ms(time_steps(e2e_step), ws, dev)
        serial_ms = slowest_rank_ms(time_steps(e2e_serial_step), ws, dev)
        # one more, untimed step with events between the calls: where the e2e time goes
        pev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        e2e_step(pev)
        torch.cuda.synchronize(dev)
        for i, name in enumerate(e2e_phase_ms):
            e2e_phase_ms[name] = pev[i].elapsed_time(pev[i + 1])
        found_h.zero_()
        stager.close()
        h2d = pairs_h.numel() * 8 + queries_h.numel() * 8 + erase_h.numel() * 8
        d2h = vals_h.numel() * 4 + found_h.numel()
        link = link_bandwidth(pairs_h, pairs, stream, dev)
        # the link bound of one step: every input byte up, every result byte down, both directions at once
        link_ms = max(h2d / link["h2d_gbs"], d2h / link["d2h_gbs"]) / 1e6
        link.update({"bound_ms": link_ms, "frac": link_ms / e2e_ms})
        e2e = {"value": ops_per_step * ws / (e2e_ms * 1e-3) / 1e6, "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
               "api": f"sg_unordered_*_host (pipelined, 2^{args.e2e_chunk_log2}-element chunks, {args.e2e_buffers} "
                      f"buffers, sg_stager_set_inputs_ready)", "link": link,
               "phases_ms": e2e_phase_ms, "phases_host_ms": e2e_host_ms, "inputs_ready": True,
               "ordered_uploads": {"value": ops_per_step * ws / (ordered_ms * 1e-3) / 1e6, "ms_per_step": ordered_ms},
               "serial_copies": {"value": ops_per_step * ws / (serial_ms * 1e-3) / 1e6, "ms_per_step": serial_ms}}

    # ---------------- roofline of the dominant kernel
    med = {k: statistics.median(v) for k, v in phase_ms.items()}
    counts = {"insert": n, "find": n_q, "erase": n_e}
    dominant = max(["insert", "find", "erase"], key=lambda k: med[k])
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    alg_bytes = BYTES_PER_OP[dominant] * counts[dominant]
    achieved = alg_bytes / (med[dominant] * 1e-3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "dram_traffic.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get(dominant)
        except (ValueError, AttributeError):
            traffic = None
    phase_kernels = {"insert": "k_part_scatter + k_ordered_staged<insert> (input chunks staged in shared memory by "
                               "bulk copies; + the gated direct k_insert, which exits at once unless the scatter "
                               "left elements out); partitioned bulk insert, chosen automatically at this size",
                     "find": "k_find", "erase": "k_part_scatter + k_ordered_staged<erase> (+ the gated direct k_erase); "
                                                 "partitioned bulk erase, chosen automatically at this size"}
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "frac_of_nominal": achieved / NOMINAL_HBM_GBS, "traffic": traffic,
                "traffic_source": "committed profile profiles/dram_traffic.json (ncu DRAM bytes of the same phase "
                                  "from the launch list of this command; not measured in this run)",
                "kernel": dominant, "kernels": phase_kernels[dominant], "peak_source": peak_src,
                "bytes_per_op": BYTES_PER_OP[dominant],
                "per_kernel": {k: {"ms": med[k], "mops": counts[k] / (med[k] * 1e-3) / 1e6,
                                   "gbs": BYTES_PER_OP[k] * counts[k] / (med[k] * 1e-3) / 1e9,
                                   "frac": BYTES_PER_OP[k] * counts[k] / (med[k] * 1e-3) / 1e9 / peak}
                               for k in counts}}
    if ceiling is not None:
        # keys (queries) per second of each phase against the random-read ceiling: one group line per key
        ceiling["per_kernel_frac"] = {k: counts[k] / (med[k] * 1e-3) / ceiling["reads_per_s"] for k in counts}
        roofline["access_ceiling"] = ceiling

    others = None
    if rank == 0 and ws == 1 and not args.no_other_configs:
        vs.close()
        vs = None
        others = other_configs(args)

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu_baseline:
        mops, kind, used, sample, _, _ = cpu_sample_run(1, keys_log2=CPU_BASELINE_KEYS_LOG2, reps=1)
        cpu = {"value": mops, "unit": UNIT, "cores": used, "kind": kind, "sample": sample,
               "std_unordered_map": std_map_line(CPU_BASELINE_KEYS_LOG2)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": f"voxel-block unordered_map<uint64_t,uint32_t>, capacity 2^{args.keys_log2 + 1}, "
                                   f"2^{args.keys_log2} keys; clear+insert+find(70% hits)+erase(25%) per step",
                       "capacity": cap, "keys": n, "finds": n_q, "erases": n_e, "parallelism": "replicas" if ws > 1 else "single",
                       "l2": "inputs larger than L2 (no flush)"},
            "phases_ms": med,
            "guard": {"checked": "sizes after each call; found flags and values of all queries; final contents",
                      "insert_launches": guard["insert_launches"], "erase_launches": guard["erase_launches"]},
            "roofline": roofline,
            "cpu_baseline": cpu,
            "e2e": e2e,
            "gpu_launches": launches,
            "clocks": clocks,
            "other_configs": others,
        }
        print(json.dumps(line), flush=True)
    if vs is not None:
        vs.close()
    if ws > 1:
        torch.distributed.destroy_process_group()


def batched_cpu_sample(threads: int, n_tables: int = 256) -> dict:
    """The reference (or the oracle restatement) on the first n_tables tables of the many-small-tables
    workload: per table createDeviceObject(capacity), insert of its keys, contains of its queries."""
    import oracle as O
    from stdgpu_gb300 import batch_bench

    counts, caps, keys, queries, offsets = batch_bench.make_workload()
    kind = "reference" if O.ref_available() else "port"
    if kind == "reference":
        O.ref_set_threads(threads)
        make = lambda c: O.RefTable(O.SET_U64, int(c))
    else:
        threads = 1
        make = lambda c: O.PortTable(O.SET_U64, int(c))
    secs, ops, hits = 0.0, 0, 0
    for t in range(n_tables):
        a, b = int(offsets[t]), int(offsets[t + 1])
        tab = make(caps[t])
        t0 = time.perf_counter()
        tab.insert(keys[a:b])
        f = tab.contains(queries[a:b])
        secs += time.perf_counter() - t0
        hits += int(f.sum())
        ops += 2 * (b - a)
        tab.close()
    return {"value": ops / secs / 1e6, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": f"the first {n_tables} of the 4096 tables ({ops // 2} keys): insert + contains per table, "
                      f"wall time of the calls (table creation excluded); {hits} hits"}


def other_configs(args) -> dict:
    """The other benchmark configurations, each run once on this GPU after the voxel step, so that one
    invocation records them all: the L2-resident small set (with the reference's CPU time of the same
    configuration), the 4096 many-small-tables step (batched and graph forms against the plain per-table
    calls from a C++ loop), the served request stream (server against serial plain calls), the large
    mixed workload (capacity-2^30 map at three loads, vector, deque, bitset), and the device calls and custom
    key types through the C++ API (one thread per key inside a caller's kernel).  A part that fails reports
    why instead of its numbers."""
    import torch

    from stdgpu_gb300 import batch_bench, device_bench, large_bench, serve_bench, small_bench

    def small():
        r = small_bench.run(steps=20, warmup=5)
        out = {"value": r["graph_mops"], "unit": UNIT, "ms_per_step": r["graph_ms"], "detail": r,
               "roofline": {"bound": "l2", "note": "the 13.7 MB table stays in the 129 MB L2; HBM fraction not "
                                                   "meaningful, launch overhead and L2 latency bound the step"}}
        cpu = []
        for th in (1, os.cpu_count() or 1):
            mops, kind, used, phases, secs = small_cpu_run(th)
            cpu.append({"value": mops, "unit": UNIT, "cores": used, "kind": kind, "step_s": secs,
                        "sample": "the full small configuration (2^20 keys, capacity 2^21): insert + contains + "
                                  "erase wall time"})
        out["cpu_baseline"] = cpu
        return out

    def batched():
        r = batch_bench.run(steps=max(args.steps, 5), warmup=max(args.warmup, 3))
        return {"value": r["graph_mops"], "unit": UNIT, "ms_per_step": r["graph_ms"],
                "plain_calls": {"value": r["plain_mops"], "ms_per_step": r["plain_ms"],
                                "driver": "C++ loop over the C ABI, 3 calls per table per step"},
                "speedup_vs_plain": r["speedup_graph"], "detail": r,
                "cpu_baseline": batched_cpu_sample(1)}

    def serve():
        r = serve_bench.run(n_requests=args.requests)
        sat, ul = r["saturated"], r["under_load"]
        return {"value": sat["server_keys_per_s"] / 1e6, "unit": "M keys/s",
                "serial_plain_calls": {"value": sat["serial_keys_per_s"] / 1e6, "unit": "M keys/s",
                                       "driver": r["serial_driver"]},
                "speedup_vs_serial": sat["speedup"], "speedup_ceiling": r["ceiling"]["speedup_ceiling"],
                "p50_us": ul["server_p50_us"], "p99_us": ul["server_p99_us"],
                "serial_p50_us": ul["serial_p50_us"], "serial_p99_us": ul["serial_p99_us"], "detail": r}

    def large():
        r = large_bench.run(full=True)
        return {"value": r["map"][-2]["find_mops"], "unit": UNIT, "detail": r,
                "note": "value: find M keys/s of the capacity-2^30 map at 0.9 load; per part in detail"}

    def device_calls():
        r = device_bench.run(keys_log2=24)
        if not r["checks_pass"]:
            raise RuntimeError(f"device_bench checks failed: {json.dumps(r)[:300]}")
        m = r["parts"][0]
        return {"value": m["find_gkeys_s"] * 1e3, "unit": UNIT, "detail": r["parts"],
                "note": "value: device find M keys/s of unordered_map<uint64_t,uint32_t> with 2^24 keys, capacity "
                        "2^25 (one thread per key in the caller's kernel); custom-key voxel sets in detail"}

    out = {}
    for name, fn in (("small", small), ("batched", batched), ("serve", serve), ("large", large),
                     ("device_calls", device_calls)):
        t0 = time.perf_counter()
        try:
            out[name] = fn()
        except Exception as ex:  # one configuration's failure never costs the headline its line
            out[name] = {"unavailable": f"{type(ex).__name__}: {str(ex)[:300]}"}
        out[name]["wall_s"] = time.perf_counter() - t0
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
    return out


def batched_arm(args):
    """Many small tables: plain per-table calls vs one batched launch vs a CUDA graph (one GPU)."""
    from stdgpu_gb300 import batch_bench
    r = batch_bench.run(steps=args.steps, warmup=args.warmup)
    line = {"metric": "many-small-tables clear+insert+contains Mops/s", "value": r["graph_mops"], "unit": UNIT,
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": r["graph_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": "4096 unordered_set<uint64_t>, lognormal counts (median 2048, sigma 1.5, "
                                   "64..262144), capacity bit_ceil(2 count), contains 50% hits"},
            "batched": r}
    print(json.dumps(line), flush=True)


def serve_arm(args):
    """Request stream over 256 resident maps: the native server vs serial plain calls (one GPU)."""
    from stdgpu_gb300 import serve_bench
    r = serve_bench.run(n_requests=args.requests)
    small = serve_bench.run(n_requests=4 * args.requests, min_n=1 << 10, max_n=1 << 14)
    line = {"metric": "served request stream keys/s and p50/p99 latency", "value": r["saturated"]["server_keys_per_s"],
            "unit": "keys/s", "n_gpus": 1, "steps": 1, "warmup": 0, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u64", "data": "synthetic",
            "config": {"workload": "256 unordered_map<uint64_t,uint64_t>, capacity log-uniform 2^16..2^24; requests "
                                   "insert 40% / find 50% / erase 10%, log-uniform 1K..4M keys, Zipf(0.99) over 2^30; "
                                   "HBM budget 120 GB"},
            "serve": r, "serve_small_requests": small}
    print(json.dumps(line), flush=True)


def large_arm(args):
    """Capacity-2^30 map at 0.5/0.75/0.9 load with Zipf batches, plus vector / deque / bitset (one GPU)."""
    from stdgpu_gb300 import large_bench
    r = large_bench.run(full=True)
    line = {"metric": "large mixed workload Mops/s", "value": r["map"][-2]["find_mops"], "unit": UNIT, "n_gpus": 1,
            "steps": 1, "warmup": 0, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic",
            "config": {"workload": "unordered_map<uint64_t,uint32_t> capacity 2^30 at 0.5/0.75/0.9 load, 2^24-key Zipf(0.99) "
                                   "insert/find batches over 2^34; vector push_back 2^28 threads 30%; deque 2^26 mixed "
                                   "ops; bitset count 2^33 bits"},
            "large": r}
    print(json.dumps(line), flush=True)


def small_arm(args):
    """unordered_set<uint32_t> capacity 2^21, 2^20 keys: an L2-resident table, eager and CUDA-graph steps."""
    from stdgpu_gb300 import small_bench
    r = small_bench.run(steps=max(args.steps, 20), warmup=max(args.warmup, 5))
    line = {"metric": "small-table clear+insert+contains+erase Mops/s", "value": r["graph_mops"], "unit": UNIT,
            "n_gpus": 1, "steps": max(args.steps, 20), "warmup": max(args.warmup, 5), "ms_per_step": r["graph_ms"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32", "data": "synthetic",
            "config": {"workload": "unordered_set<uint32_t>, capacity 2^21, 2^20 uniform keys; contains 50% hits; "
                                   "erase half; step replayed as one CUDA graph (table resident in L2)"},
            "small": r}
    print(json.dumps(line), flush=True)


def device_arm(args):
    """Device calls (one thread per key in a caller's kernel) and custom key types, through the C++ API."""
    from stdgpu_gb300 import device_bench
    r = device_bench.run(keys_log2=args.keys_log2 if args.keys_log2 <= 26 else 26)
    m = r["parts"][0] if r["parts"] else {}
    line = {"metric": "device-call find M keys/s", "value": m.get("find_gkeys_s", 0.0) * 1e3, "unit": UNIT, "n_gpus": 1,
            "steps": 1, "warmup": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
            "data": "synthetic",
            "config": {"workload": "device insert / find / erase of unordered_map<uint64_t,uint32_t> (distinct random "
                                   "keys, capacity 2 x keys); 3 x int16 and 3 x int32 voxel sets with the spatial hash: "
                                   "bulk insert, device contains (hits, misses), device insert, bulk erase"},
            "device_calls": r}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        reference_arm(args)
    elif args.workload == "device":
        device_arm(args)
    elif args.workload == "large":
        large_arm(args)
    elif args.workload == "small":
        small_arm(args)
    elif args.workload == "serve":
        serve_arm(args)
    elif args.workload == "batched":
        batched_arm(args)
    else:
        native_arm(args)


if __name__ == "__main__":
    main()

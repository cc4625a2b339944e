"""Served request stream workload: continuous batching vs serial plain calls (one GB300).

256 live unordered_map<uint64_t, uint64_t> tables, capacity log-uniform in 2^16..2^24.  Each request
picks a table uniformly and is an insert (40 %), find (50 %) or erase (10 %) of a log-uniform 1K..4M
keys drawn Zipf(0.99) over a 2^30-rank universe per table (rank -> key by a seeded bijective 64-bit
mix, salted per table); values are a hash of the key.  HBM budget 120 GB.  Measured:

* saturated throughput: all requests submitted back to back, server vs serial plain calls (one
  request at a time, each a C-ABI call on the table's own object followed by a stream sync, driven from
  a C++ loop).  Two serial paths: `serial` starts from the admitted capacities and rehashes a table
  before an insert that needs room, by the server's growth policy; `serial_presized` runs on tables
  created at the capacities the server's tables ended with, so it never rehashes (its best case);
* the speed-up ceiling: the presized serial calls once more without synchronisation, each timed on the
  device; the device time of the requests large enough to fill the GPU on their own bounds any schedule;
* latency under load: Poisson arrivals at 80 % of the serial path's saturated request rate (the device is
  at least that busy under the serial path), p50 / p99 of submission-to-completion for the server and
  for both serial paths fed the same arrivals.
"""

from __future__ import annotations

import time
from ctypes import c_void_p

import numpy as np
import torch

from . import _native as N
from . import comparators as P
from . import containers as C
from . import server as S
from . import workloads as W


def zipf_ranks(rng, n, universe=2**30, s=0.99):
    u = rng.random(n)
    a = 1.0 - s
    return np.floor((1.0 + u * (universe ** a - 1.0)) ** (1.0 / a)).astype(np.uint64)


def make_stream(n_tables=256, n_requests=600, seed=0, min_n=1 << 10, max_n=1 << 22, cap_log2=(16, 24)):
    rng = np.random.default_rng(seed)
    caps = np.exp(rng.uniform(np.log(2 ** cap_log2[0]), np.log(2 ** cap_log2[1]), size=n_tables)).astype(np.int64)
    salts = W.mix64(np.arange(n_tables, dtype=np.uint64) + np.uint64(12345))
    reqs = []
    for _ in range(n_requests):
        t = int(rng.integers(0, n_tables))
        op = int(rng.choice([S.INSERT, S.FIND, S.ERASE], p=[0.4, 0.5, 0.1]))
        n = int(np.exp(rng.uniform(np.log(min_n), np.log(max_n))))
        keys = W.mix64(zipf_ranks(rng, n) ^ salts[t])
        reqs.append((t, op, keys))
    return caps, reqs


def stage(reqs):
    """Device buffers of every request (keys, values for inserts, outputs)."""
    out = []
    for t, op, keys in reqs:
        k = torch.from_numpy(keys.view(np.int64)).cuda()
        v = torch.from_numpy(W.mix64(keys).view(np.int64)).cuda() if op == S.INSERT else None
        ov = torch.empty(len(keys), dtype=torch.int64, device="cuda") if op == S.FIND else None
        of = torch.empty(len(keys), dtype=torch.uint8, device="cuda")
        out.append((t, op, k, v, ov, of))
    torch.cuda.synchronize()
    return out


def run_server(caps, staged, arrivals=None, budget=120 << 30, policy: dict | None = None):
    srv = S.server(key="u64", mapped="u64", budget_bytes=budget, n_streams=8, n_slots=16)
    if policy:
        srv.set_policy(**policy)
    for t, c in enumerate(caps):
        if srv.admit(t, int(c)) != N.SG_OK:
            raise RuntimeError("budget too small for the initial tables")
    t0 = time.perf_counter()
    if arrivals is None:
        # every request is ready at once: one call submits them all
        tickets = srv.submit_many(staged)
    else:
        tickets = []
        for i, (t, op, k, v, ov, of) in enumerate(staged):
            due = t0 + arrivals[i]
            while time.perf_counter() < due:
                pass
            tickets.append(srv.submit(t, op, k, v, ov, of))
    statuses = [srv.wait(tk) for tk in tickets]
    wall = time.perf_counter() - t0
    st = srv.stats()
    st["latency_us"] = [srv.latency_us(tk) for tk in tickets]
    final_caps = []
    for t in range(len(caps)):
        v = srv.table_view(t)
        final_caps.append(int(v.bucket_count))
    sizes = [srv.table_size(t) for t in range(len(caps))]
    srv.close()
    return wall, st, statuses, final_caps, sizes


def run_serial(caps, staged, arrivals=None, sync_each: bool = True, kernel_times: bool = False, grow: bool = False):
    """The plain path from a C++ loop over the C ABI (comparators.serial_replay): each request is one call on
    its table's own object; with sync_each the stream is synchronised after every request (the serial
    plain path), without it the calls run back to back (the device time of the same kernels).  With grow
    the loop rehashes a table before an insert that needs room, by the server's policy (the tables then
    start at the admitted capacities); without it the tables must already be large enough."""
    tables = [C.unordered_map.createDeviceObject(int(c), key="u64", mapped="u64") for c in caps]
    for t in tables:
        t.set_excess_accounting(False)  # the server's tables: keys until no slot is free, tile kernels
    reqs = [N.sg_request(t, op, k.numel(), k.data_ptr(), v.data_ptr() if v is not None else None,
                         ov.data_ptr() if ov is not None else None, of.data_ptr())
            for t, op, k, v, ov, of in staged]
    torch.cuda.synchronize()
    lat, ker, wall, rehashes = P.serial_replay(tables, reqs, arrivals, sync_each=sync_each,
                                               kernel_times=kernel_times,
                                               grow_kind=N.MAP_U64_U64 if grow else None)
    sizes = [tb.size() for tb in tables]
    for tb in tables:
        C.unordered_base.destroyDeviceObject(tb)
    return wall, lat, ker, sizes, rehashes


def ceiling(staged, kernel_us, serial_s: float, direct_keys: int = 1 << 16) -> dict:
    """Upper bound of the speed-up any scheduler can reach over the serial path on this stream.  A request
    of at least direct_keys keys fills the GPU by itself (each such launch is a persistent grid over every
    SM), so overlapping it with other work cannot shorten it much; the device time of those requests,
    measured back to back, is a floor under any schedule's wall time, and serial / floor bounds the
    speed-up.  Small requests are assumed to overlap completely."""
    n = np.array([k.numel() for _, _, k, _, _, _ in staged])
    big = n >= direct_keys
    k_us = np.asarray(kernel_us, dtype=np.float64)
    floor_s = float(k_us[big].sum()) * 1e-6
    return {
        "direct_keys": direct_keys,
        "keys_in_large_requests": float(n[big].sum() / n.sum()),
        "large_requests": int(big.sum()),
        "device_time_all_s": float(k_us.sum()) * 1e-6,
        "device_time_large_s": floor_s,
        "serial_s": serial_s,
        "speedup_ceiling": serial_s / floor_s if floor_s > 0 else None,
    }


def tail_requests(staged, lat_server, lat_serial, k: int = 8) -> dict:
    """The k slowest requests under load on each path: operation, keys and both latencies (microseconds)."""
    ops = {S.INSERT: "insert", S.FIND: "find", S.ERASE: "erase"}
    ls, lp = np.asarray(lat_server, dtype=np.float64), np.asarray(lat_serial, dtype=np.float64)

    def rows(order):
        return [{"op": ops[staged[i][1]], "keys": int(staged[i][2].numel()), "server_us": round(float(ls[i]), 1),
                 "serial_us": round(float(lp[i]), 1)} for i in order[:k]]

    return {"server": rows(np.argsort(-ls)), "serial": rows(np.argsort(-lp))}


def run(n_requests=600, seed=0, load=0.8, min_n=1 << 10, max_n=1 << 22, policy: dict | None = None) -> dict:
    """The server against two serial plain paths on the same request stream: `serial` starts from the
    admitted capacities and grows its tables by the server's policy (what a plain caller must do), and
    `serial_presized` runs on tables created at the capacities the server's tables ended with (no rehash
    at all: the best case of the plain path, which needs the stream's future)."""
    caps, reqs = make_stream(n_requests=n_requests, seed=seed, min_n=min_n, max_n=max_n)
    staged = stage(reqs)
    keys_total = int(sum(len(r[2]) for r in reqs))
    # saturated server (also gives the capacity each table grows to)
    wall_srv, st_sat, statuses, final_caps, sizes_srv = run_server(caps, staged, policy=policy)
    refused = sum(1 for s in statuses if s != N.SG_OK)
    wall_ser, _, _, sizes_ser, ser_rehashes = run_serial(caps, staged, grow=True)
    wall_pre, _, _, sizes_pre, _ = run_serial(final_caps, staged)
    # the presized calls back to back (no host synchronisation), each timed on the device: the ceiling
    wall_stream, _, ker_us, _, _ = run_serial(final_caps, staged, sync_each=False, kernel_times=True)
    bound = ceiling(staged, ker_us, wall_pre)
    bound["stream_no_sync_s"] = wall_stream
    # Poisson arrivals at `load` x the serial path's saturated request rate: the device is at least that busy
    # under the serial path, and every path sees the same arrivals
    rate = load * len(staged) / wall_ser
    rng = np.random.default_rng(seed + 1)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, size=len(staged)))
    wall_srv_l, st_load, _, _, _ = run_server(caps, staged, arrivals, policy=policy)
    wall_ser_l, lat_ser_load, _, _, _ = run_serial(caps, staged, arrivals, grow=True)
    wall_pre_l, lat_pre_load, _, _, _ = run_serial(final_caps, staged, arrivals)
    pct = lambda a, q: float(np.percentile(a, q))
    return {
        "request_keys": [min_n, max_n],
        "tables": len(caps), "requests": len(staged), "keys": keys_total,
        "refused_requests": refused, "rehashes": st_sat["rehashes"], "serial_rehashes": ser_rehashes,
        "hbm_used_bytes": st_sat["hbm_used_bytes"],
        "saturated": {
            "server_s": wall_srv, "serial_s": wall_ser, "serial_presized_s": wall_pre,
            "server_keys_per_s": keys_total / wall_srv, "serial_keys_per_s": keys_total / wall_ser,
            "serial_presized_keys_per_s": keys_total / wall_pre,
            "server_requests_per_s": len(staged) / wall_srv, "serial_requests_per_s": len(staged) / wall_ser,
            "speedup": wall_ser / wall_srv, "speedup_vs_presized": wall_pre / wall_srv,
            "waves": st_sat["waves"], "launches": st_sat["launches"],
            "grow_host_us": st_sat.get("grow_host_us"), "max_grow_host_us": st_sat.get("max_grow_host_us"),
            "grow_create_us": st_sat.get("grow_create_us"),
        },
        "policy": policy or "default",
        "under_load": {
            "arrival_rate_per_s": rate, "load_vs_serial_capacity": load,
            "server_p50_us": st_load["p50_us"], "server_p99_us": st_load["p99_us"],
            "serial_p50_us": pct(lat_ser_load, 50), "serial_p99_us": pct(lat_ser_load, 99),
            "serial_presized_p50_us": pct(lat_pre_load, 50), "serial_presized_p99_us": pct(lat_pre_load, 99),
            "server_wall_s": wall_srv_l, "serial_wall_s": wall_ser_l, "serial_presized_wall_s": wall_pre_l,
            "server_keys_per_s": keys_total / wall_srv_l, "serial_keys_per_s": keys_total / wall_ser_l,
        },
        "ceiling": bound,
        "tail": tail_requests(staged, st_load["latency_us"], lat_ser_load),
        "tail_vs_presized": tail_requests(staged, st_load["latency_us"], lat_pre_load),
        "serial_driver": "C++ loop over the C ABI (stdgpu_gb300/comparators/plain_calls.cpp)",
        "final_sizes_agree": bool(sizes_srv == sizes_ser == sizes_pre),
    }


if __name__ == "__main__":
    # the server alone on a chosen stream, e.g. for a profiler capture of its segmented launches:
    #   python -m stdgpu_gb300.serve_bench --tables 64 --requests 400 --max-log2 14 --cap-log2 16 20
    import argparse
    import json

    ap = argparse.ArgumentParser()
    ap.add_argument("--tables", type=int, default=256)
    ap.add_argument("--requests", type=int, default=600)
    ap.add_argument("--min-log2", type=int, default=10)
    ap.add_argument("--max-log2", type=int, default=22)
    ap.add_argument("--cap-log2", type=int, nargs=2, default=[16, 24])
    a = ap.parse_args()
    caps, reqs = make_stream(n_tables=a.tables, n_requests=a.requests, min_n=1 << a.min_log2, max_n=1 << a.max_log2,
                             cap_log2=tuple(a.cap_log2))
    staged = stage(reqs)
    wall, st, statuses, _, _ = run_server(caps, staged)
    keys = int(sum(len(r[2]) for r in reqs))
    print(json.dumps({"server_s": wall, "keys_per_s": keys / wall, "launches": st["launches"],
                      "refused": sum(1 for x in statuses if x != N.SG_OK)}))

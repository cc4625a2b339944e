"""Served request stream: every result in the mix equals the serial replay (alone, one request after
another) of the same request sequence, plus budget refusal and growth under the budget."""

import numpy as np
import pytest
import torch

import oracle as O
import stdgpu_gb300 as sg
from stdgpu_gb300 import _native as N
from stdgpu_gb300 import server as S
from stdgpu_gb300 import workloads as W

from gpu_util import dev, host, per_key_success

pytestmark = pytest.mark.gpu


def zipf_keys(rng, n, universe, s=0.99):
    """Zipf(s) ranks over [1, universe] by inverse CDF of the continuous approximation, mixed to keys."""
    u = rng.random(n)
    a = 1.0 - s
    ranks = np.floor((1.0 + u * (universe ** a - 1.0)) ** (1.0 / a)).astype(np.uint64)
    return W.mix64(ranks)


def make_requests(seed, n_tables, n_req, max_n):
    rng = np.random.default_rng(seed)
    reqs = []
    for _ in range(n_req):
        t = int(rng.integers(0, n_tables))
        op = int(rng.choice([S.INSERT, S.FIND, S.ERASE], p=[0.4, 0.5, 0.1]))
        n = int(np.exp(rng.uniform(np.log(16), np.log(max_n))))
        keys = zipf_keys(rng, n, 2**20)
        vals = W.mix64(keys ^ np.uint64(0x9E3779B97F4A7C15))
        reqs.append((t, op, keys, vals))
    return reqs


def maximal_runs(reqs):
    """Per table, indices of maximal runs of consecutive same-operation requests (submission order)."""
    runs = []
    current = {}
    for i, (t, op, _, _) in enumerate(reqs):
        if t in current and reqs[current[t][-1]][1] == op:
            current[t].append(i)
        else:
            if t in current:
                runs.append(current[t])
            current[t] = [i]
    runs.extend(current.values())
    return runs


def test_served_results_equal_serial_replay():
    n_tables = 6
    reqs = make_requests(1, n_tables, 160, 20000)
    srv = S.server(key="u64", mapped="u64", budget_bytes=8 << 30, n_streams=4, n_slots=8)
    caps = [1 << 15] * n_tables
    for t in range(n_tables):
        assert srv.admit(t, caps[t]) == N.SG_OK
    staged = [(dev(keys), dev(vals) if op == S.INSERT else None) for _, op, keys, vals in reqs]
    outs = [srv.new_outputs(len(keys)) for _, _, keys, _ in reqs]
    torch.cuda.synchronize()
    tickets = []
    # the first half queues while the scheduler is paused, so it coalesces; the rest streams in live
    srv.pause(True)
    for i, (t, op, keys, vals) in enumerate(reqs):
        if i == len(reqs) // 2:
            srv.pause(False)
        ov, of = outs[i]
        tickets.append(srv.submit(t, op, staged[i][0], staged[i][1], ov if op == S.FIND else None, of))
    for tk in tickets:
        assert srv.wait(tk) == N.SG_OK
    st = srv.stats()
    assert st["requests_done"] == len(reqs)
    # serial replay, one request at a time, on the oracle
    # the server grows tables under its budget instead of refusing; the replay tables are large enough
    # never to refuse
    ports = [O.PortTable(O.MAP_U64_U64, 1 << 21) for _ in caps]
    serial_flags = []
    for i, (t, op, keys, vals) in enumerate(reqs):
        if op == S.INSERT:
            serial_flags.append(ports[t].insert(keys, vals, flags=True))
        elif op == S.ERASE:
            serial_flags.append(ports[t].erase(keys, flags=True))
        else:
            pv, pf = ports[t].find(keys)
            serial_flags.append(pf)
            gv = host(outs[i][0], np.uint64)
            gf = outs[i][1].cpu().numpy()
            assert np.array_equal(gf, pf), i
            assert np.array_equal(gv[pf == 1], pv[pf == 1]), i
    # inserts / erases: per key, successes summed over each maximal same-operation run agree
    for run in maximal_runs(reqs):
        if reqs[run[0]][1] == S.FIND:
            continue
        keys = np.concatenate([reqs[i][2] for i in run])
        got = np.concatenate([outs[i][1].cpu().numpy() for i in run])
        want = np.concatenate([serial_flags[i] for i in run])
        assert per_key_success(keys, got) == per_key_success(keys, want), run
    for t in range(n_tables):
        assert srv.table_size(t) == ports[t].size()
    assert st["waves"] < len(reqs)  # requests were coalesced
    srv.close()


def test_budget_refuses_admission_and_growth():
    g = sg.geometry_for(N.MAP_U64_U64, 1 << 16)
    budget = 3 * g.storage_bytes + g.storage_bytes // 2
    srv = S.server(key="u64", mapped="u64", budget_bytes=budget, n_streams=2, n_slots=4)
    assert srv.admit(0, 1 << 16) == N.SG_OK
    assert srv.admit(1, 1 << 16) == N.SG_OK
    assert srv.admit(2, 1 << 16) == N.SG_OK
    assert srv.admit(3, 1 << 16) == N.SG_ERR_BUDGET
    # table 0 would need to grow past the budget: refused, nothing spilled, table unchanged
    keys = np.arange(1, 200001, dtype=np.uint64)
    _, of = srv.new_outputs(len(keys))
    tk = srv.submit(0, S.INSERT, dev(keys), dev(keys), None, of)
    assert srv.wait(tk) == N.SG_ERR_BUDGET
    assert srv.stats()["refused_budget"] == 1
    assert srv.table_size(0) == 0
    # a request that fits still runs
    tk = srv.submit(0, S.INSERT, dev(keys[:1000]), dev(keys[:1000]), None, of[:1000])
    assert srv.wait(tk) == N.SG_OK and srv.table_size(0) == 1000
    srv.close()


def test_growth_under_budget_keeps_contents():
    srv = S.server(key="u64", mapped="u64", budget_bytes=4 << 30, n_streams=2, n_slots=4)
    assert srv.admit(7, 1 << 10) == N.SG_OK
    rng = np.random.default_rng(5)
    all_keys = []
    for _ in range(6):
        keys = rng.integers(1, 2**62, size=3000, dtype=np.uint64)
        all_keys.append(keys)
        tk = srv.submit(7, S.INSERT, dev(keys), dev(keys * np.uint64(3)), None, None)
        assert srv.wait(tk) == N.SG_OK
    assert srv.stats()["rehashes"] >= 1
    everything = np.unique(np.concatenate(all_keys))
    ov, of = srv.new_outputs(len(everything))
    tk = srv.submit(7, S.FIND, dev(everything), None, ov, of)
    assert srv.wait(tk) == N.SG_OK
    assert of.cpu().numpy().sum() == len(everything)
    assert np.array_equal(host(ov, np.uint64), everything * np.uint64(3))
    assert srv.table_size(7) == len(everything)
    srv.close()


def test_growth_moves_out_of_band_keys_and_skips_erased_slots():
    """A grow rebuilds the table on the device: erased slots stay behind, the two out-of-band keys (all
    ones and all ones minus one) move with their values, and the latency of every request is reported."""
    srv = S.server(key="u64", mapped="u64", budget_bytes=4 << 30, n_streams=2, n_slots=4)
    assert srv.admit(3, 1 << 10) == N.SG_OK
    rng = np.random.default_rng(11)
    keys = rng.integers(1, 2**62, size=700, dtype=np.uint64)
    keys[:2] = [np.uint64(2**64 - 1), np.uint64(2**64 - 2)]
    port = O.PortTable(O.MAP_U64_U64, 1 << 16)
    tickets = [srv.submit(3, S.INSERT, dev(keys), dev(keys ^ np.uint64(5)), None, None)]
    port.insert(keys, keys ^ np.uint64(5))
    gone = keys[1:300:3]  # one out-of-band key and about a hundred others
    tickets.append(srv.submit(3, S.ERASE, dev(gone), None, None, None))
    port.erase(gone)
    more = rng.integers(1, 2**62, size=3000, dtype=np.uint64)
    tickets.append(srv.submit(3, S.INSERT, dev(more), dev(more ^ np.uint64(5)), None, None))
    port.insert(more, more ^ np.uint64(5))
    assert all(srv.wait(t) == N.SG_OK for t in tickets)
    assert srv.stats()["rehashes"] >= 1
    assert all(srv.latency_us(t) > 0 for t in tickets)
    probe = np.concatenate([keys, more, rng.integers(1, 2**62, size=500, dtype=np.uint64)])
    ov, of = srv.new_outputs(len(probe))
    tk = srv.submit(3, S.FIND, dev(probe), None, ov, of)
    assert srv.wait(tk) == N.SG_OK
    want_vals, want_found = port.find(probe)
    got_found = of.cpu().numpy().astype(bool)
    assert np.array_equal(got_found, want_found.astype(bool))
    assert np.array_equal(host(ov, np.uint64)[got_found], want_vals[got_found])
    assert srv.table_size(3) == port.size()
    srv.close()


def test_back_to_back_grows_release_replaced_storage_for_the_budget():
    """Two grows of one table in one burst: the storage the first grow replaced is still held when the second
    needs room, and the budget only allows the second once it is released."""
    c = 1 << 12
    geo = [sg.geometry_for(N.MAP_U64_U64, c << k) for k in range(3)]
    s = [g.storage_bytes for g in geo]
    budget = s[1] + s[2] + s[0] // 2  # the three never fit at once
    srv = S.server(key="u64", mapped="u64", budget_bytes=budget, n_streams=2, n_slots=4)
    assert srv.admit(0, c) == N.SG_OK
    rng = np.random.default_rng(12)
    ms0 = geo[0].max_size
    k1 = rng.integers(1, 2**62, size=ms0 * 9 // 10, dtype=np.uint64)  # past 85 % of the first max_size
    k2 = rng.integers(1, 2**62, size=ms0, dtype=np.uint64)  # then past 85 % of the second's
    tickets = srv.submit_many([(0, S.INSERT, dev(k1), dev(k1), None, None),
                               (0, S.FIND, dev(k1), None, *srv.new_outputs(len(k1))),
                               (0, S.INSERT, dev(k2), dev(k2), None, None)])
    assert [srv.wait(t) for t in tickets] == [N.SG_OK] * 3
    st = srv.stats()
    assert st["rehashes"] == 2 and st["refused_budget"] == 0
    assert st["hbm_used_bytes"] <= budget
    assert srv.table_size(0) == len(np.unique(np.concatenate([k1, k2])))
    srv.close()


def test_idle_table_past_half_grows_ahead_and_keeps_contents():
    """An insert that leaves a table more than half full, with nothing else queued for it, lets the idle table
    grow to the next doubling before another insert arrives; its contents stay, and so does the order of what
    is submitted meanwhile."""
    import time as _time

    c = 1 << 12
    g0 = sg.geometry_for(N.MAP_U64_U64, c)
    srv = S.server(key="u64", mapped="u64", budget_bytes=4 << 30, n_streams=2, n_slots=4)
    assert srv.admit(5, c) == N.SG_OK
    rng = np.random.default_rng(13)
    keys = np.unique(rng.integers(1, 2**62, size=g0.max_size * 6 // 10, dtype=np.uint64))
    tk = srv.submit(5, S.INSERT, dev(keys), dev(keys + np.uint64(1)), None, None)
    assert srv.wait(tk) == N.SG_OK
    deadline = _time.time() + 10.0
    while srv.stats()["rehashes"] < 1 and _time.time() < deadline:
        _time.sleep(0.01)
    assert srv.stats()["rehashes"] == 1  # grown ahead, with no second insert submitted
    assert srv.table_view(5).bucket_count > g0.bucket_count
    ov, of = srv.new_outputs(len(keys))
    tk = srv.submit(5, S.FIND, dev(keys), None, ov, of)
    assert srv.wait(tk) == N.SG_OK
    assert of.cpu().numpy().all()
    assert np.array_equal(host(ov, np.uint64), keys + np.uint64(1))
    assert srv.table_size(5) == len(keys)
    # switched off, a table left the same way stays as it is
    srv.set_grow_ahead(False)
    assert srv.admit(6, c) == N.SG_OK
    tk = srv.submit(6, S.INSERT, dev(keys), dev(keys), None, None)
    assert srv.wait(tk) == N.SG_OK
    _time.sleep(0.2)
    assert srv.stats()["rehashes"] == 1
    assert srv.table_view(6).bucket_count == g0.bucket_count
    srv.close()

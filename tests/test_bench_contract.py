"""bench.py's reference arm (host code only) prints one JSON line with every key of the benchmark contract."""

import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_reference_arm_line_has_the_contract_keys():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--steps", "1", "--warmup", "0"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [x for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
              "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["unit"] == "Mops/s" and d["scaling"] == "weak"
    assert {"workload", "capacity", "keys", "finds", "erases"} <= set(d["config"])
    # ms_per_step is the measured step of the sample the config names (one step here: exactly the value)
    c = d["config"]
    ops = c["keys"] + c["finds"] + c["erases"]
    assert abs(ops / (d["ms_per_step"] * 1e3) - d["value"]) <= 1e-6 * d["value"]
    cb = d["cpu_baseline"]
    assert {"value", "unit", "cores", "kind", "sample"} <= set(cb) and cb["kind"] in ("reference", "port")
    # the std::unordered_map sanity line (one host thread, same sample)
    sm = cb["std_unordered_map"]
    assert "unavailable" in sm or (sm["kind"] == "std::unordered_map" and sm["value"] > 0 and sm["cores"] == 1)
    e = d["e2e"]
    assert e["value"] == d["value"] and e["unit"] == d["unit"]
    assert e["h2d_bytes_per_step"] == 0 and e["d2h_bytes_per_step"] == 0

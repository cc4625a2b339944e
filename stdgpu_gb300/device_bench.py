"""Device calls and custom key types, measured through the C++ API (``stdgpu_gb300/device_bench.cu``).

The program is compiled against the built library on first use (a few seconds) and run in a child
process; each part prints one JSON line with its rates and whether its checks passed.
"""

from __future__ import annotations

import json
import subprocess
from pathlib import Path

from . import build as B

SRC = Path(__file__).resolve().parent / "device_bench.cu"
EXE = B.OUT / "device_bench"


def build() -> Path:
    lib = B.library_path()
    deps = [SRC, lib] + list(B.INCLUDE.rglob("*.cuh")) + list(B.INCLUDE.rglob("*.h"))
    if EXE.exists() and all(p.stat().st_mtime <= EXE.stat().st_mtime for p in deps):
        return EXE
    tmp = EXE.with_name(EXE.name + ".tmp")
    B._run([B.nvcc(), *B.ARCH_FLAGS, "-O3", "-std=c++17", "-lineinfo", "-I", str(B.INCLUDE), str(SRC),
            "-L", str(lib.parent), "-lstdgpu_gb300", f"-Xlinker=-rpath={lib.parent}", "-o", str(tmp)])
    tmp.replace(EXE)
    return EXE


def run(keys_log2: int = 24, timeout: float = 600.0) -> dict:
    """Runs every part at 2^keys_log2 keys; returns {"parts": [...], "checks_pass": bool}."""
    exe = build()
    r = subprocess.run([str(exe), str(keys_log2)], capture_output=True, text=True, timeout=timeout)
    parts = [json.loads(line) for line in r.stdout.splitlines() if line.startswith("{")]
    parts = parts[1:]  # the first line is a 4096-key warm-up of the device-call map
    ok = r.returncode == 0 and len(parts) == 3 and all(p.get("checks_pass") for p in parts)
    return {"parts": parts, "checks_pass": ok, "returncode": r.returncode,
            "stderr": r.stderr[-500:] if r.returncode != 0 else ""}


if __name__ == "__main__":
    import sys
    print(json.dumps(run(int(sys.argv[1]) if len(sys.argv) > 1 else 24), indent=1))

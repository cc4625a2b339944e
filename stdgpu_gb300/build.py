"""Builds the product library ``stdgpu_gb300/_lib/libstdgpu_gb300.so`` for sm_103a.

Plain ``nvcc`` (no CMake, no torch extension machinery): one object per
translation unit, compiled in parallel, linked into one shared library with a
C ABI (``include/stdgpu_gb300.h``).  The same recipe runs on x86_64 and on the
aarch64 GPU host.
"""

from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OUT = PKG / "_lib"
INCLUDE = ROOT / "include"
LIB_NAME = "libstdgpu_gb300.so"

# translation units of the product library
SOURCES = ["unordered.cu", "containers.cu", "batch.cu", "server.cu", "staged.cu", "snapshot.cu", "diag.cu"]

ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden"]


def nvcc() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    p = Path(cuda) / "bin" / "nvcc"
    return str(p) if p.exists() else (shutil.which("nvcc") or "nvcc")


def _run(cmd: list[str]) -> str:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return r.stdout + r.stderr


# the plain-call comparators (host C++ over the C ABI; stdgpu_gb300/comparators)
COMPARATORS_SRC = PKG / "comparators" / "plain_calls.cpp"
COMPARATORS_LIB = "libsg_plain_calls.so"


def build_comparators() -> Path:
    """Compile the plain-call comparator library against the product library (g++, static CUDA runtime)."""
    out = OUT / COMPARATORS_LIB
    lib = library_path()
    if out.exists() and out.stat().st_mtime >= max(COMPARATORS_SRC.stat().st_mtime, lib.stat().st_mtime,
                                                    (INCLUDE / "stdgpu_gb300.h").stat().st_mtime):
        return out
    cuda = Path(os.environ.get("CUDA_HOME", "/usr/local/cuda"))
    tmp = OUT / (COMPARATORS_LIB + ".tmp")
    _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fvisibility=hidden", "-I", str(INCLUDE),
          "-I", str(cuda / "include"), str(COMPARATORS_SRC), "-o", str(tmp), "-L", str(OUT), "-lstdgpu_gb300",
          "-Wl,-rpath,$ORIGIN", "-L", str(cuda / "lib64"), "-lcudart_static", "-ldl", "-lpthread", "-lrt"])
    os.replace(tmp, out)
    return out


def _deps() -> list[Path]:
    return list(CSRC.glob("*.cu")) + list(CSRC.glob("*.cuh")) + list(INCLUDE.rglob("*.h")) + \
        list(INCLUDE.rglob("*.cuh")) + [Path(__file__)]


def library_path() -> Path:
    return OUT / LIB_NAME


def is_current() -> bool:
    lib = library_path()
    if not lib.exists() or os.environ.get("STDGPU_GB300_NVCC_FLAGS"):
        return False
    t = lib.stat().st_mtime
    deps = _deps() + ([TUNING] if TUNING.exists() else [])
    return all(p.stat().st_mtime <= t for p in deps)


# launch shapes of the single-table kernels chosen by stdgpu_gb300/autotune_single.py (compile-time macros)
TUNING = PKG / "tuning" / "single_table.json"


def tuned_flags() -> list[str]:
    """-D flags of the recorded best single-table launch shapes (none when no record exists)."""
    if not TUNING.exists():
        return []
    import json
    best = json.loads(TUNING.read_text()).get("best", {})
    return [f"-D{k}={int(v)}" for k, v in sorted(best.items())]


def build(force: bool = False, verbose_ptxas: bool = False, flags: list[str] | None = None,
          out_lib: Path | None = None) -> Path:
    """Compile every translation unit for sm_103a and link the shared library.  `flags` replaces the recorded
    launch shapes (autotuning builds its candidates this way, into `out_lib`)."""
    if flags is None and out_lib is None and not force and is_current():
        build_comparators()
        return library_path()
    OUT.mkdir(exist_ok=True)
    extra = ["-Xptxas", "-v"] if verbose_ptxas else []
    extra += tuned_flags() if flags is None else list(flags)
    # optional extra compiler flags, e.g. -DSG_BULK_MIN_BLOCKS=3
    extra += os.environ.get("STDGPU_GB300_NVCC_FLAGS", "").split()
    cmds = []
    objs = []
    obj_dir = OUT if out_lib is None else out_lib.parent / (out_lib.stem + "_obj")
    obj_dir.mkdir(parents=True, exist_ok=True)
    for src in SOURCES:
        obj = obj_dir / (Path(src).stem + ".o")
        objs.append(obj)
        cmds.append([nvcc(), *ARCH_FLAGS, *NVCC_FLAGS, *extra, "-I", str(INCLUDE), "-I", str(CSRC),
                     "-c", str(CSRC / src), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=len(cmds)) as ex:
        logs = list(ex.map(_run, cmds))
    target = library_path() if out_lib is None else out_lib
    tmp = target.parent / (target.name + ".tmp")
    _run([nvcc(), *ARCH_FLAGS, "-shared", "-o", str(tmp), *[str(o) for o in objs], "-lcudart"])
    os.replace(tmp, target)
    if verbose_ptxas:
        (obj_dir / "ptxas.log").write_text("\n".join(logs))
    if out_lib is None:
        build_comparators()
    return target


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv))

"""Build recipe for the two CPU checkers under ``oracle/`` (test infrastructure).

1. ``oracle/_build/liboracle_port.so`` -- the plain-C restatement in ``port.c``.
2. ``oracle/_ref/libsgref.so`` -- the reference library itself (stdgpu 1.3.0,
   OpenMP backend) plus ``ref_driver.cpp``, compiled directly with g++ from its
   own five translation units (no CMake):
     src/stdgpu/impl/{device,iterator,memory}.cpp, src/stdgpu/openmp/impl/{device,memory}.cpp
   The reference's CMake writes one ``config.h`` from ``config.h.in``
   (src/stdgpu/CMakeLists.txt:27-29); this recipe writes the same eight defines
   for the OpenMP backend with 32-bit ``index_t`` and contract checks off
   (Release defaults, src/stdgpu/CMakeLists.txt:10-22).  Thrust comes from the
   CUDA toolkit's CCCL headers.

The reference tree is read from the ``ref_root`` argument of ``build_reference``,
else from ``$STDGPU_REFERENCE``, else from REFERENCE_MOUNT (where the build
container mounts the reference checkout, read-only); it is staged into the
git-ignored ``oracle/_ref/src`` so that the same recipe can rebuild the checker on
a machine where only the staged copy exists (the GPU host).  Nothing here is part
of the product library.
"""

from __future__ import annotations

import os
import platform
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

HERE = Path(__file__).resolve().parent
# the read-only reference checkout of the build container, the last place this recipe looks
REFERENCE_MOUNT = Path("/root/reference")
REF_OUT = HERE / "_ref"
PORT_OUT = HERE / "_build"
STAGE = REF_OUT / "src"

REF_TUS = [
    "stdgpu/impl/device.cpp",
    "stdgpu/impl/iterator.cpp",
    "stdgpu/impl/memory.cpp",
    "stdgpu/openmp/impl/device.cpp",
    "stdgpu/openmp/impl/memory.cpp",
]

CONFIG_H = """#ifndef STDGPU_CONFIG_H
#define STDGPU_CONFIG_H
namespace stdgpu
{
#define STDGPU_VERSION_MAJOR 1
#define STDGPU_VERSION_MINOR 3
#define STDGPU_VERSION_PATCH 0
#define STDGPU_VERSION_STRING "1.3.0"
#define STDGPU_BACKEND STDGPU_BACKEND_OPENMP
#define STDGPU_BACKEND_DIRECTORY openmp
#define STDGPU_BACKEND_NAMESPACE openmp
#define STDGPU_BACKEND_MACRO_NAMESPACE OPENMP
#define STDGPU_ENABLE_CONTRACT_CHECKS 0
#define STDGPU_USE_32_BIT_INDEX 1
}
#endif
"""


def _cccl_include() -> str:
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    arch = "sbsa-linux" if platform.machine() in ("aarch64", "arm64") else "x86_64-linux"
    return f"{cuda}/targets/{arch}/include/cccl"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"command failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def _newer(target: Path, sources: list[Path]) -> bool:
    if not target.exists():
        return False
    t = target.stat().st_mtime
    return all(s.stat().st_mtime <= t for s in sources if s.exists())


def build_port() -> Path:
    """Compile the C restatement into a shared library."""
    PORT_OUT.mkdir(exist_ok=True)
    so = PORT_OUT / "liboracle_port.so"
    srcs = [HERE / "port.c", HERE / "port.h"]
    if not _newer(so, srcs):
        _run(["gcc", "-std=c11", "-O2", "-fPIC", "-shared", "-Wall", "-Wextra",
              str(HERE / "port.c"), "-o", str(so), "-lm"])
    return so


def stage_reference(ref_root: Path) -> None:
    """Copy the reference headers and its five OpenMP-backend TUs into oracle/_ref/src."""
    src = ref_root / "src" / "stdgpu"
    dst = STAGE / "stdgpu"
    if dst.exists():
        shutil.rmtree(dst)
    for p in src.rglob("*"):
        rel = p.relative_to(src)
        parts = rel.parts
        if parts and parts[0] in ("cuda", "hip"):
            continue  # other backends are not compiled
        if p.is_dir() or p.suffix not in (".h", ".cuh", ".cpp"):
            continue
        out = dst / rel
        out.parent.mkdir(parents=True, exist_ok=True)
        shutil.copy2(p, out)
    (dst / "config.h").write_text(CONFIG_H)


def build_reference(jobs: int = 8, ref_root: Path | str | None = None) -> Path | None:
    """Stage (when the reference tree is present) and compile libsgref.so."""
    if ref_root is None:
        ref_root = os.environ.get("STDGPU_REFERENCE") or REFERENCE_MOUNT
    ref_root = Path(ref_root)
    if (ref_root / "src" / "stdgpu").is_dir():
        stage_reference(ref_root)
    if not (STAGE / "stdgpu" / "config.h").exists():
        return None
    so = REF_OUT / "libsgref.so"
    driver = HERE / "ref_driver.cpp"
    tus = [STAGE / t for t in REF_TUS] + [driver]
    if _newer(so, tus + [HERE / "build_oracle.py"]) and so.stat().st_mtime >= (STAGE / "stdgpu" / "config.h").stat().st_mtime:
        return so
    flags = ["g++", "-std=c++17", "-O2", "-fPIC", "-fopenmp", "-DNDEBUG",
             "-DTHRUST_DEVICE_SYSTEM=THRUST_DEVICE_SYSTEM_OMP",
             "-I", str(STAGE), "-isystem", _cccl_include(), "-w"]
    objs = []
    cmds = []
    for tu in tus:
        obj = REF_OUT / (tu.name.replace(".cpp", "") + ("_omp" if "openmp" in str(tu) else "") + ".o")
        objs.append(obj)
        cmds.append(flags + ["-c", str(tu), "-o", str(obj)])
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        list(ex.map(_run, cmds))
    _run(["g++", "-shared", "-fopenmp", "-o", str(so)] + [str(o) for o in objs])
    return so


def main() -> int:
    port = build_port()
    print(f"port: {port}")
    ref = build_reference()
    print(f"reference: {ref if ref else 'not available (no staged reference tree)'}")
    return 0


if __name__ == "__main__":
    sys.exit(main())

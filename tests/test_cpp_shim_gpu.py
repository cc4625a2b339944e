"""The C++ API with the reference's names (include/stdgpu_gb300/stdgpu.cuh), used by a program that
runs the reference's own test scenarios with native device calls inside user kernels."""

import subprocess
from pathlib import Path

import pytest

import stdgpu_gb300
from stdgpu_gb300 import build as B

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "shim_test.cu"
CUSTOM = ROOT / "tests" / "cpp" / "custom_key_test.cu"
WIDE = ROOT / "tests" / "cpp" / "wide_key_test.cu"
OUT = ROOT / "tests" / "cpp" / "_build"


def _compile(flags=(), src=SRC):
    OUT.mkdir(exist_ok=True)
    lib = stdgpu_gb300.library_path()
    exe = OUT / src.stem
    cmd = [B.nvcc(), *B.ARCH_FLAGS, "-std=c++17", "-O2", *flags, "-I", str(ROOT / "include"), str(src),
           "-L", str(lib.parent), "-lstdgpu_gb300", f"-Xlinker=-rpath={lib.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_for_sm103a():
    """CPU part: the header compiles with the test program (no device needed)."""
    stdgpu_gb300.load()
    _compile()


@pytest.mark.gpu
def test_shim_reference_scenarios_on_gpu():
    stdgpu_gb300.load()
    exe = _compile()
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASS" in r.stdout


def test_custom_key_program_compiles_for_sm103a():
    stdgpu_gb300.load()
    _compile(src=CUSTOM)


@pytest.mark.gpu
def test_custom_key_types_with_user_hash_on_gpu():
    """3 x int16 keys with the spatial hash: bulk and device calls, heterogeneous lookup, the README's
    neighbour-update kernel, all against std::unordered_set / std::unordered_map."""
    stdgpu_gb300.load()
    exe = _compile(src=CUSTOM)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASS" in r.stdout


def test_wide_key_program_compiles_for_sm103a():
    stdgpu_gb300.load()
    _compile(src=WIDE)


@pytest.mark.gpu
def test_wide_keys_and_nontrivial_types_on_gpu():
    """The reference's nontrivial-type table (3 x int32 key with a destructor, empty mapped type) and its
    clear_nontrivial scenario, 16-byte keys on every bit pattern, 16-byte mapped values, mapped destructors
    counted through erase / clear / destroy, refusal at max_size(), against the host containers."""
    stdgpu_gb300.load()
    exe = _compile(src=WIDE)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASS" in r.stdout

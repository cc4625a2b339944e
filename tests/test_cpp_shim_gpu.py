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
WIDE_GOLDEN = ROOT / "tests" / "cpp" / "wide_golden_test.cu"
ROUTING = ROOT / "tests" / "cpp" / "routing_check.cu"
CHURN = ROOT / "tests" / "cpp" / "device_churn_test.cu"
KEY_EQUAL = ROOT / "tests" / "cpp" / "key_equal_test.cu"
ALLOCATOR = ROOT / "tests" / "cpp" / "allocator_test.cu"
GOLDEN = ROOT / "tests" / "golden"
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


def test_wide_golden_program_compiles_for_sm103a():
    stdgpu_gb300.load()
    _compile(src=WIDE_GOLDEN)


def write_fixture(npz, out_dir):
    """The arrays of a table_vec3i32 fixture as raw little-endian files for the C++ replay."""
    import numpy as np
    g = np.load(npz)
    meta = np.array([g["capacity"], g["max_size"], g["bucket_count"], g["size_after_insert"],
                     g["size_after_erase"]], np.int64)
    meta.tofile(out_dir / "meta.bin")
    for name in ("keys", "queries", "found", "erase", "final_keys", "buckets", "insert_flags", "erase_flags",
                 "values", "found_values", "final_values"):
        if name in g.files:
            np.ascontiguousarray(g[name]).tofile(out_dir / f"{name}.bin")


@pytest.mark.gpu
@pytest.mark.parametrize("kind,mode", [(8, "set"), (9, "map")])
def test_wide_keys_replay_reference_fixtures(tmp_path, kind, mode):
    """unordered_set<vec3i32> / unordered_map<vec3i32, uint64_t> with the spatial hash on the wide tables:
    geometry, bucket(), sizes, find answers and values, final contents and per-key device outcomes equal
    what the reference itself recorded (tests/golden/table_vec3i32_<kind>.npz)."""
    stdgpu_gb300.load()
    exe = _compile(src=WIDE_GOLDEN)
    write_fixture(GOLDEN / f"table_vec3i32_{kind}.npz", tmp_path)
    r = subprocess.run([str(exe), str(tmp_path), mode], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASS" in r.stdout


def test_element_types_route_to_the_intended_storage():
    """Compile-time: precompiled kinds for integer keys with the default hash, the word-keyed path for other
    keys of up to 8 bytes, the wide tables for the rest (static_asserts in tests/cpp/routing_check.cu)."""
    stdgpu_gb300.load()
    _compile(src=ROUTING)


def test_device_churn_program_compiles_for_sm103a():
    stdgpu_gb300.load()
    _compile(src=CHURN)


@pytest.mark.gpu
def test_device_insert_erase_churn_reuses_erased_slots(tmp_path):
    """Device-only insert / erase churn on tiny tables for hundreds of launches: per-key outcomes and sizes
    equal a std::unordered_set / std::unordered_map model after every launch, no insert of an absent key is
    refused below max_size() (erased slots are reused), racing inserts and erases of one key keep at most
    one copy.  The set churn's launches are then replayed on the oracle restatement (and on the reference
    library where it is built) launch by launch, with equal per-key outcomes and sizes."""
    import numpy as np

    import oracle as O
    from gpu_util import per_key_success

    stdgpu_gb300.load()
    exe = _compile(src=CHURN)
    r = subprocess.run([str(exe), str(tmp_path)], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASS" in r.stdout
    cap, launches = np.fromfile(tmp_path / "header.bin", dtype=np.int64)
    meta = np.fromfile(tmp_path / "meta.bin", dtype=np.int32).reshape(-1, 2)
    keys = np.fromfile(tmp_path / "keys.bin", dtype=np.uint64)
    ok = np.fromfile(tmp_path / "ok.bin", dtype=np.uint8)
    assert len(meta) == launches
    tables = [O.PortTable(O.SET_U64, int(cap))]
    if O.ref_available():
        O.ref_set_threads(1)
        tables.append(O.RefTable(O.SET_U64, int(cap)))
    pos = 0
    for n, n_ins in meta:
        k, f = keys[pos: pos + n], ok[pos: pos + n]
        pos += n
        for t in tables:
            fi = t.insert(k[:n_ins], flags=True)
            fe = t.erase(k[n_ins:], flags=True)
            assert per_key_success(k[:n_ins], f[:n_ins]) == per_key_success(k[:n_ins], fi)
            assert per_key_success(k[n_ins:], f[n_ins:]) == per_key_success(k[n_ins:], fe)
    sizes = {t.size() for t in tables}
    assert len(sizes) == 1
    for t in tables:
        t.close()


def test_key_equal_program_compiles_for_sm103a():
    stdgpu_gb300.load()
    _compile(src=KEY_EQUAL)


@pytest.mark.gpu
def test_keys_compare_with_key_equal_on_gpu():
    """Keys equal under KeyEqual are one key (a tagged key compared by one field; float keys, +0.0 == -0.0):
    bulk and device calls against std::unordered_set / std::unordered_map with the same Hash and KeyEqual."""
    stdgpu_gb300.load()
    exe = _compile(src=KEY_EQUAL)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASS" in r.stdout


def test_allocator_program_compiles_for_sm103a():
    stdgpu_gb300.load()
    _compile(src=ALLOCATOR)


@pytest.mark.gpu
def test_user_allocator_holds_every_block_on_gpu():
    """createDeviceObject(capacity, allocator) with a counting device allocator on the three storage paths:
    every block from it, tables working, every block returned by destroyDeviceObject."""
    stdgpu_gb300.load()
    exe = _compile(src=ALLOCATOR)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL PASS" in r.stdout

"""CPU checks of the drop-in boundary: the C-ABI library loads and exports every symbol that
include/kfr_capi.h declares, the declarations match the reference's C API surface, and the planner's pure
host logic behaves.  No GPU call is made here."""
import ctypes
import os
import re

import pytest

import kfr_gb300 as k

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# Every entry point of the reference's C API (include/kfr/capi.h:116-736): 79 names, including the
# KFR_MANAGED_ALLOCATION helpers (capi.h:178-193).
REFERENCE_DFT_API = [
    "kfr_version_string", "kfr_version", "kfr_enabled_archs", "kfr_current_arch", "kfr_last_error",
    "kfr_allocate", "kfr_allocate_aligned", "kfr_deallocate", "kfr_reallocate", "kfr_reallocate_aligned",
    "kfr_add_ref", "kfr_release", "kfr_allocated_size",
] + [f"kfr_dft_{op}_{p}" for p in ("f32", "f64") for op in (
    "create_plan", "create_2d_plan", "create_3d_plan", "create_md_plan", "dump", "get_size", "get_temp_size",
    "execute", "execute_inverse", "delete_plan")] + [f"kfr_dft_real_{op}_{p}" for p in ("f32", "f64") for op in (
        "create_plan", "create_2d_plan", "create_3d_plan", "create_md_plan", "dump", "get_size", "get_temp_size",
        "execute", "execute_inverse", "delete_plan")] + [f"kfr_dct_{op}_{p}" for p in ("f32", "f64") for op in (
            "create_plan", "dump", "get_size", "get_temp_size", "execute", "execute_inverse", "delete_plan")] + [
    f"kfr_filter_{op}_{p}" for p in ("f32", "f64") for op in (
        "create_fir_plan", "create_convolution_plan", "create_iir_plan", "process", "reset", "delete_plan")]


@pytest.fixture(scope="module")
def L():
    if not os.path.exists(k.LIB_PATH):
        k_build = __import__("kfr_gb300.build", fromlist=["build"])
        k_build.build()
    return k.lib()


def test_header_declares_reference_api():
    declared = set(k.declared_symbols())
    missing = [s for s in REFERENCE_DFT_API if s not in declared]
    assert not missing, missing


def test_library_exports_every_declared_symbol(L):
    out = os.popen(f"nm -D --defined-only {k.LIB_PATH}").read()
    exported = set(line.split()[-1] for line in out.splitlines() if line.strip())
    declared = k.declared_symbols()
    assert declared, "no declarations parsed"
    missing = [s for s in declared if s not in exported]
    assert not missing, missing
    # nothing but the C API leaks out of the library
    extra = [s for s in exported if not s.startswith("kfr_") and not s.startswith("_init") and not s.startswith("_fini")]
    assert not extra, extra[:10]


def test_reference_header_types_match():
    """ABI-relevant constants: pack-format values and the default alignment (include/kfr/capi.h:165-200)."""
    text = open(os.path.join(ROOT, "include", "kfr_capi.h")).read()
    assert re.search(r"Perm\s*=\s*0", text) and re.search(r"CCs\s*=\s*1", text)
    assert "#define KFR_DEFAULT_ALIGNMENT 64" in text
    for t in ("KFR_DFT_PLAN_F32", "KFR_DFT_REAL_PLAN_F64", "KFR_DCT_PLAN_F32", "KFR_FILTER_F64", "KFR_FILTER_C32"):
        assert f"KFR_OPAQUE_STRUCT({t})" in text


def test_version_and_error_convention(L):
    assert L.kfr_version() == 70001
    assert k.version_string().startswith("KFR 7.0.1")
    assert L.kfr_enabled_archs() == b"sm_103a"
    # NULL handles never crash: size queries return 0 and leave a message
    assert L.kfr_dft_get_size_f32(None) == 0
    assert b"NULL" in L.kfr_last_error()
    L.kfr_dft_delete_plan_f32(None)  # NULL is allowed (capi.h:366)
    assert L.kfr_last_error() == b""


def test_host_allocation_without_gpu(L):
    p = L.kfr_allocate(1000)
    assert p and p % 64 == 0
    ctypes.memset(p, 1, 1000)
    L.kfr_deallocate(p)
    p = L.kfr_allocate_aligned(100, 4096)
    assert p % 4096 == 0
    L.kfr_deallocate(p)
    assert L.kfr_last_error() == b""


def test_reference_api_has_79_entry_points():
    assert len(set(REFERENCE_DFT_API)) == 79


def test_managed_allocation(L):
    """kfr_reallocate / kfr_reallocate_aligned / kfr_add_ref / kfr_release / kfr_allocated_size follow the
    reference's managed allocation (include/kfr/meta/memory.hpp:58-140): contents survive a reallocation,
    a block lives until its last reference is released, and the size query returns the requested size."""
    p = L.kfr_allocate(100)
    assert L.kfr_allocated_size(p) == 100
    ctypes.memmove(p, bytes(range(100)), 100)
    q = L.kfr_reallocate(p, 300)  # grows: the first 100 bytes are kept
    assert q and q % 64 == 0 and L.kfr_allocated_size(q) == 300
    assert ctypes.string_at(q, 100) == bytes(range(100))
    r = L.kfr_reallocate_aligned(q, 40, 4096)  # shrinks: the first 40 bytes are kept
    assert r % 4096 == 0 and L.kfr_allocated_size(r) == 40
    assert ctypes.string_at(r, 40) == bytes(range(40))
    assert L.kfr_add_ref(r) == r  # two references now
    L.kfr_release(r)
    assert L.kfr_allocated_size(r) == 40  # still alive after one release
    L.kfr_release(r)  # last reference: freed
    assert L.kfr_last_error() == b""
    assert not L.kfr_reallocate(None, 0)
    s = L.kfr_reallocate(None, 16)  # NULL pointer: plain allocation
    assert s and L.kfr_allocated_size(s) == 16
    assert not L.kfr_reallocate(s, 0)  # size 0: released, NULL returned
    assert L.kfr_last_error() == b""
    assert not L.kfr_allocate_aligned(16, 0)  # alignment 0 or above 32768: NULL, as in the reference
    assert not L.kfr_allocate_aligned(16, 65536)
    assert b"alignment" in L.kfr_last_error()
    big = L.kfr_allocate(1 << 20)  # large blocks are registered (pinned) where a GPU is present
    assert L.kfr_allocated_size(big) == 1 << 20
    L.kfr_deallocate(big)
    assert L.kfr_last_error() == b""


def test_out_of_scope_filters_report_errors(L):
    assert not L.kfr_filter_create_iir_plan_f32(None, 0)
    assert b"not part of the GPU DFT path" in L.kfr_last_error()
    assert not L.kfr_filter_create_iir_plan_f64(None, 0)
    assert b"not part of the GPU DFT path" in L.kfr_last_error()


def test_cpp_api_header_compiles_against_reference_style_code():
    """include/kfr_dft.hpp mirrors KFR's C++ DFT interface; tests/cpp/test_cpp_api.cpp is written against it
    the way reference users write against kfr/dft.hpp.  Compile-only here (no GPU)."""
    import subprocess

    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "test_cpp_api.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_c_header_compiles_as_c():
    """The C ABI header is valid C (C99, _Complex element types)."""
    import subprocess
    import tempfile

    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "t.c")
        with open(src, "w") as f:
            f.write('#include "kfr_capi.h"\nint main(void) { KFR_DFT_PLAN_F32* p = kfr_dft_create_plan_f32(8);'
                    ' kfr_dft_delete_plan_f32(p); return 0; }\n')
        r = subprocess.run(["gcc", "-std=c99", "-fsyntax-only", "-I", os.path.join(ROOT, "include"), src],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr

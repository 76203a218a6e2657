"""CPU checks of the C-ABI library: it loads, exports every declared symbol, and
its pure host logic (argument checks, workspace sizing) behaves.  No compute call
is made here; those run in the gpu-marked tests."""
import os
import re
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HDR_C = os.path.join(ROOT, "include", "xss_gpu.h")


def _declared_c_functions():
    text = open(HDR_C).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = set(re.findall(r"\b((?:xss_|keyvalue_qsort_)\w+)\s*\(", text))
    return sorted(n for n in names if not n.startswith("xss_stream"))


def test_library_loads_and_reports_version(xss):
    L = xss.lib()
    assert b"sm_103a" in L.xss_version()
    assert L.xss_strerror(0) == b"ok"
    assert L.xss_strerror(3) == b"device-side bounded wait expired"


def test_every_c_symbol_in_header_is_exported(xss):
    names = _declared_c_functions()
    assert len(names) >= 30, names
    L = xss.lib()
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_reference_c_symbols_present(xss):
    # lib/x86simdsort.cpp:298-339
    L = xss.lib()
    for k in ("float", "uint64", "int32", "uint32"):
        for v in ("uint32", "uint64"):
            assert hasattr(L, f"keyvalue_qsort_{k}_{v}")


def test_cxx_template_specialisations_exported(xss):
    """include/x86simdsort.h declares the reference's templates; the library must
    define them for the reference's type set (lib/x86simdsort.cpp:167-293)."""
    out = subprocess.run(["nm", "-DC", "--defined-only", xss.LIB_PATH], check=True,
                         stdout=subprocess.PIPE, text=True).stdout
    count = lambda fn: len(re.findall(r"x86simdsort::%s<[^>]*>\(" % fn, out))  # noqa: E731
    for fn in ("qsort", "qselect", "partial_qsort", "argsort", "argselect"):
        assert count(fn) == 9, (fn, count(fn))   # 8 integer/float types + _Float16
    for fn in ("keyvalue_qsort", "keyvalue_select", "keyvalue_partial_sort"):
        assert count(fn) == 36, (fn, count(fn))


def test_workspace_sizes_are_host_logic(xss):
    ws = xss.workspace_size
    # one-CTA path needs no scratch
    assert ws("qsort", "float32", 4096) == 0
    big = ws("qsort", "float32", 1 << 20)
    assert big >= (1 << 20) * 4
    assert ws("qsort", "float32", 1 << 22) > big
    assert ws("keyvalue_qsort", "int64", 1 << 20, val_dtype="uint64") > \
        ws("qsort", "int64", 1 << 20)
    assert ws("argsort", "float64", 1 << 20) > ws("qsort", "float64", 1 << 20)
    assert ws("qselect", "float32", 1 << 20) > 0


def test_invalid_arguments_rejected_before_any_device_work(xss):
    L = xss.lib()
    a = np.zeros(8, np.float32)
    assert L.xss_qsort(99, a.ctypes.data, 8, 0, 0) == 1           # bad dtype
    assert L.xss_qsort(5, None, 8, 0, 0) == 1                     # null with n > 1
    assert L.xss_qsort(5, a.ctypes.data, (1 << 40) + 1, 0, 0) == 6  # above XSS_MAX_N
    assert L.xss_keyvalue_qsort(0, 99, a.ctypes.data, a.ctypes.data, 8, 0, 0) == 1  # bad value type
    assert L.xss_keyvalue_qsort(6, -1, a.ctypes.data, a.ctypes.data, 8, 0, 0) == 1  # bad value type
    assert L.xss_gpu_object_qsort(a.ctypes.data, 4, 16, 0, 0, 0, 0, None, 0, None) == 5  # u16 key
    assert L.xss_gpu_object_qsort(a.ctypes.data, 4, 16, 12, 6, 0, 0, None, 0, None) == 1  # past end
    assert L.xss_qsort(5, a.ctypes.data, 1, 0, 0) == 0            # n <= 1 is a no-op
    assert L.xss_qselect(5, a.ctypes.data, 0, 0, 0, 0) == 0       # empty select


def test_headers_compile_and_link_without_a_gpu(xss, tmp_path):
    """The C header is plain C, and the C++ drop-in and static headers compile
    and link a caller program against the library (nothing is run here)."""
    inc = os.path.join(ROOT, "include")
    c_src = tmp_path / "abi.c"
    c_src.write_text('#include "xss_gpu.h"\nint main(void) { return xss_strerror(0) ? 0 : 1; }\n')
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", inc, "-c", str(c_src), "-o",
                    str(tmp_path / "abi.o")], check=True)
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    pkg = os.path.dirname(xss.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O0", "-I", inc, "-I", os.path.join(cuda_home, "include"),
                    os.path.join(ROOT, "tests", "cxx", "test_api.cpp"), "-o",
                    str(tmp_path / "test_api"), "-L", pkg, "-lxss_gb300", "-L",
                    os.path.join(cuda_home, "lib64"), "-lcudart"], check=True)
    assert (tmp_path / "test_api").exists()

"""C++ drop-in header compiled and run on the GPU; bounded device waits end in
XSS_ETIMEOUT and leave the context usable."""
import os
import subprocess

import numpy as np
import pytest

from xss_arrays import assert_same_sorted, get_array, ref_sorted

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_cxx_api_program(xss, cuda):
    pkg = os.path.dirname(xss.LIB_PATH)
    exe = os.path.join(HERE, "_build", "test_api")
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    cuda_home = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), "-I",
                    os.path.join(cuda_home, "include"), os.path.join(HERE, "cxx", "test_api.cpp"),
                    "-o", exe, "-L", pkg, "-lxss_gb300", "-L", os.path.join(cuda_home, "lib64"),
                    "-lcudart", f"-Wl,-rpath,{pkg}"], check=True)
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=300)
    assert r.returncode == 0, r.stdout
    assert "cxx api ok" in r.stdout


@pytest.mark.parametrize("which", [0, 1])
def test_bounded_wait_times_out_and_context_survives(xss, cuda, which):
    import ctypes
    f = xss.lib().xss_gpu_selftest_bounded_wait
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_uint, ctypes.c_void_p]
    assert f(which, 2000, None) == 3  # XSS_ETIMEOUT
    xss.stream_status()               # the library's own error word is untouched
    x = get_array("random", "float32", 100_000, 1)
    y = x.copy()
    xss.qsort(y)
    assert_same_sorted(y, ref_sorted(x), "sort after a timed-out wait")


def test_rank_order_of_shared_atomics(xss, cuda):
    """The radix pass ranks each key by the result of its shared-memory count
    atomic; that is stable only if same-address atomics of one warp
    instruction return in lane order.  The library's self test checks it on
    this device over about 300 million collisions of many patterns."""
    import ctypes
    f = xss.lib().xss_gpu_selftest_rank_order
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.POINTER(ctypes.c_ulonglong), ctypes.c_void_p]
    v = ctypes.c_ulonglong(123)
    assert f(ctypes.byref(v), None) == 0
    assert v.value == 0

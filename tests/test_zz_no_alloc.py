"""xss_gpu_qsort_noalloc: the allocation-free sort, through the C ABI.

It exists for callers that may not allocate device memory when they sort (an
allocator or out-of-memory handler, a plugin whose host owns all device
memory, a fixed-budget real-time loop).  Its output must equal xss_gpu_qsort's
for the same input, call after call, although every call reuses one fixed
scratch array.  This file is collected last so that a stop-at-first-failure
run has already run every other test; it also passes on its own in a fresh
process.  The first call on a device is its set-up (it loads the kernels, which
allocates); the memory test checks that later calls leave the device's free
memory unchanged.
"""
import ctypes

import numpy as np
import pytest

from xss_arrays import assert_same_sorted, get_array, ref_sorted

pytestmark = pytest.mark.gpu

MAX_N = 1 << 20
DT = {"uint16": 0, "int16": 1, "float16": 2, "uint32": 3, "int32": 4, "float32": 5,
      "uint64": 6, "int64": 7, "float64": 8}


def _noalloc(xss):
    f = xss.lib().xss_gpu_qsort_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int,
                  ctypes.c_void_p]
    return f


@pytest.mark.parametrize("dtype", ["float32", "int64", "float16", "uint32", "float64"])
def test_noalloc_matches_qsort_twice_in_a_row(xss, cuda, dtype):
    torch = cuda
    f = _noalloc(xss)
    stream = torch.cuda.Stream()
    # two calls in a row per size: the second finds the first call's data in
    # the shared scratch and must still agree with the regular entry point
    for n in (3000, 250_000, MAX_N):
        for call, seed in enumerate((1, 2)):
            shape = "mixed_special" if dtype.startswith("float") else "random"
            x = get_array(shape, dtype, n, seed=seed + 10 * n)
            for desc in (0, 1):
                a = torch.from_numpy(x.view(np.uint8).copy()).cuda()
                b = torch.from_numpy(x.view(np.uint8).copy()).cuda()
                torch.cuda.synchronize()
                rc = f(DT[dtype], a.data_ptr(), n, 1, desc, stream.cuda_stream)
                assert rc == 0, (dtype, n, call, rc)
                xss.gpu_qsort(dtype, b.data_ptr(), n, True, bool(desc), stream=stream.cuda_stream)
                xss.stream_status(stream.cuda_stream)
                ga = a.cpu().numpy().view(x.dtype)
                gb = b.cpu().numpy().view(x.dtype)
                # the tests' tolerance for sorts: identical bytes after
                # canonicalising +-0 and NaN payloads
                assert_same_sorted(ga, gb, f"noalloc vs qsort {dtype} n={n} call={call}")
                assert_same_sorted(ga, ref_sorted(x, bool(desc)), f"noalloc {dtype} n={n}")


def test_noalloc_rejects_sizes_above_its_limit(xss, cuda):
    torch = cuda
    f = _noalloc(xss)
    n = MAX_N + 1
    x = get_array("random", "float32", n, seed=3)
    a = torch.from_numpy(x.copy()).cuda()
    rc = f(DT["float32"], a.data_ptr(), n, 0, 0, None)
    assert rc == 6  # XSS_ETOOBIG
    assert np.array_equal(a.cpu().numpy(), x)  # untouched


def test_noalloc_leaves_device_free_memory_unchanged(xss, cuda):
    torch = cuda
    f = _noalloc(xss)
    stream = torch.cuda.Stream()
    cases = []
    for dtype in ("uint16", "float32", "int64"):
        for n in (3000, MAX_N):
            x = get_array("random", dtype, n, seed=7 + n)
            cases.append((dtype, n, torch.from_numpy(x.view(np.uint8).copy()).cuda()))
    # set-up call (first on this device, or a repeat when earlier tests ran)
    x0 = torch.zeros(5000, dtype=torch.float32, device="cuda")
    assert f(DT["float32"], x0.data_ptr(), 5000, 0, 0, stream.cuda_stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for _ in range(2):
        for dtype, n, a in cases:
            assert f(DT[dtype], a.data_ptr(), n, 1, 0, stream.cuda_stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    # a cudaMalloc (the library's workspace cache, a lazily loaded kernel)
    # would take at least one 2 MiB page of device memory
    assert free1 == free0, (free0, free1)

"""Host-pointer sorts of large arrays take the pipelined path (chunk copies
overlapped with chunk sorts, then merged and copied back slice by slice).
Its results must equal the device-pointer sort of the same input exactly
(both are stable where order can be told apart), from pageable and from
pinned host buffers."""
import os
import subprocess
import sys

import numpy as np
import pytest

from golden_io import DT
from xss_arrays import assert_same_sorted, bit_code, get_array

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))

N = (1 << 22) + 12345


def _pinned(torch, a):
    t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
    v = t.numpy().view(a.dtype)
    v[:] = a
    return t, v


@pytest.mark.parametrize("pinned", [False, True])
def test_keyvalue_host_pipeline_equals_device_sort(xss, cuda, pinned):
    torch = cuda
    rng = np.random.default_rng(3)
    k = rng.integers(-2**40, 2**40, N, dtype=np.int64)
    k[::7] = 12345                          # ties: the order of their values is checked
    v = np.arange(N, dtype=np.uint64)
    hold = []
    if pinned:
        tk, k_h = _pinned(torch, k)
        tv, v_h = _pinned(torch, v)
        hold += [tk, tv]
    else:
        k_h, v_h = k.copy(), v.copy()
    xss.keyvalue_qsort(k_h, v_h, False, True)
    dk = torch.from_numpy(k.copy()).cuda()
    dv = torch.from_numpy(v.view(np.int64).copy()).cuda()
    xss.gpu_keyvalue_qsort("int64", "uint64", dk.data_ptr(), dv.data_ptr(), N, False, True)
    xss.stream_status()
    assert np.array_equal(k_h, dk.cpu().numpy())
    assert np.array_equal(v_h, dv.cpu().numpy().view(np.uint64))


def test_qsort_host_pipeline_matches_oracle(xss, oracle, cuda):
    x = get_array("rand_with_nan", "float32", N, seed=21)
    got = x.copy()
    xss.qsort(got, True, False)
    want = x.copy()
    assert oracle.qsort(DT["float32"], want.ctypes.data, N, 1, 0) == 0
    assert_same_sorted(got, want, "pipelined qsort float32")


@pytest.mark.parametrize("dtype", ["float64", "uint16"])
def test_argsort_host_pipeline_is_stable_order(xss, cuda, dtype):
    x = get_array("mixed_special" if dtype == "float64" else "smallrange", dtype, N, seed=22)
    arg = xss.argsort(x, True, True)
    want = np.argsort(bit_code(x, True), kind="stable")
    assert np.array_equal(arg.astype(np.int64), want)


@pytest.mark.parametrize("chunk", ["899840", "649984", "499968"])
def test_host_pipeline_more_chunks(xss, cuda, chunk):
    # 5, 7 and 9 chunks: merge levels run between the chunk sorts and meet
    # partial blocks (a child process, as the chunk length is read once)
    env = dict(os.environ, XSS_MERGE_CHUNK=chunk)
    r = subprocess.run([sys.executable, os.path.join(HERE, "host_pipeline_cases.py")], env=env,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=900)
    assert r.returncode == 0, r.stdout[-4000:]
    assert "0 failures" in r.stdout

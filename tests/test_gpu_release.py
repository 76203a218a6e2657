"""xss_release_cached: the device memory the library keeps between calls --
the per-stream workspace of device-pointer calls made without a workspace,
and this thread's staging and pipeline buffers of host-pointer calls -- is
freed, and later calls allocate again and still sort correctly.  No
counterpart in the reference (a CPU library keeps no device memory)."""
import numpy as np
import pytest

from xss_arrays import assert_pairs_preserved, assert_same_sorted, get_array, ref_sorted

pytestmark = pytest.mark.gpu


def _fill_caches(xss, torch):
    # device-pointer sort without a workspace: the NULL stream's cached workspace
    n_dev = 1 << 24
    x = get_array("random", "float32", n_dev, 41)
    d = torch.from_numpy(x.copy()).cuda()
    xss.gpu_qsort("float32", d.data_ptr(), n_dev, False, False)
    xss.stream_status()
    assert_same_sorted(d.cpu().numpy(), ref_sorted(x), "device qsort")
    # host-pointer key-value sort of 2^23 pairs: the pipelined path's buffers
    # (keys, values and their merge partners: 4 x 64 MiB, plus a chunk workspace)
    n_host = 1 << 23
    k = get_array("random", "int64", n_host, 42)
    v = np.arange(n_host, dtype=np.uint64)
    kk, vv = k.copy(), v.copy()
    xss.keyvalue_qsort(kk, vv, False, False)
    assert_same_sorted(kk, ref_sorted(k), "host keyvalue_qsort")
    assert_pairs_preserved(k, v, kk, vv, "host keyvalue_qsort")
    # host-pointer sort below the pipeline's size: the staging buffer
    y = get_array("random", "uint32", 1 << 20, 43)
    yy = y.copy()
    xss.qsort(yy, False, False)
    assert_same_sorted(yy, ref_sorted(y), "host qsort")


def test_release_cached_frees_and_calls_still_work(xss, cuda):
    torch = cuda
    _fill_caches(xss, torch)
    torch.cuda.synchronize()
    free_before = torch.cuda.mem_get_info()[0]
    xss.release_cached()
    free_after = torch.cuda.mem_get_info()[0]
    freed = free_after - free_before
    assert freed >= 256 << 20, f"only {freed} bytes freed"
    # a second release finds nothing to free and still succeeds
    xss.release_cached()
    assert abs(torch.cuda.mem_get_info()[0] - free_after) < (64 << 20)
    # every path allocates again and sorts correctly, and the caches can be
    # released once more
    _fill_caches(xss, torch)
    xss.release_cached()

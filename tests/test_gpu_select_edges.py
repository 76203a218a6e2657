"""Selects of 32/64-bit keys on device arrays that start off a 16-byte
boundary, through the device-pointer C ABI (csrc/xss_select.cu), against the
CPU oracle's sorted order.

k far from both ends takes the out-of-place split (round 0's read copies the
keys -- and a key-value select's values -- to scratch, the split writes the
outer classes back into the caller's arrays); k near an end takes the sparse
in-place split.  Unaligned keys send round 0 down its element-by-element loop
and the value copy down its unaligned path, so both copy routes are covered.
Checked: the exact k-th element at k with the partition property, the same
multiset of keys, every (key, value) pair kept, argselect a permutation, and
the elements around the array untouched.  Reference semantics:
src/xss-common-qsort.h:607-649 (qselect_), src/xss-common-keyvaluesort.hpp:519-562
(kvselect_), src/xss-common-argsort.h:551-585 (argselect_).
"""
import numpy as np
import pytest

from golden_io import DT
from xss_arrays import (UINT, assert_is_permutation, assert_pairs_preserved,
                        assert_partitioned, assert_same_sorted, get_array, ref_sorted)

pytestmark = pytest.mark.gpu

N = 200_003
GUARD = 0x5A


def _dev(torch, host, pad):
    """Device copy of `host` starting `pad` elements into a buffer filled with GUARD bytes."""
    isz = host.itemsize
    buf = torch.full(((host.size + 8) * isz,), GUARD, dtype=torch.uint8, device="cuda")
    raw = torch.from_numpy(host.view(np.uint8).copy()).cuda()
    buf[pad * isz:(pad + host.size) * isz] = raw
    return buf, buf.data_ptr() + pad * isz


def _back(buf, host, pad):
    isz = host.itemsize
    b = buf.cpu().numpy()
    assert (b[:pad * isz] == GUARD).all() and (b[(pad + host.size) * isz:] == GUARD).all()
    return b[pad * isz:(pad + host.size) * isz].view(host.dtype).copy()


def _ks(n):
    return [5, n // 3, n // 2, n - 7]     # near an end -> sparse split; otherwise out of place


@pytest.mark.parametrize("pad", [0, 1, 3])
@pytest.mark.parametrize("dtype", ["float32", "int64", "uint32", "float64"])
def test_qselect_unaligned(xss, oracle, cuda, dtype, pad):
    x = get_array("rand_with_nan" if dtype.startswith("float") else "random", dtype, N, 11 + pad)
    srt = {}
    for desc in (False, True):
        srt[desc] = x.copy()
        assert oracle.qsort(DT[dtype], srt[desc].ctypes.data, N, 1, int(desc)) == 0
    for k in _ks(N):
        for desc in (False, True):
            buf, ptr = _dev(cuda, x, pad)
            xss.gpu_qselect(dtype, ptr, k, N, True, desc)
            xss.stream_status()
            got = _back(buf, x, pad)
            what = f"qselect {dtype} pad={pad} k={k} desc={desc}"
            assert_partitioned(got, k, srt[desc][k], desc, what)
            assert_same_sorted(ref_sorted(got), ref_sorted(x), "multiset " + what)


@pytest.mark.parametrize("pad", [0, 1, 3])
@pytest.mark.parametrize("ktype,vtype", [("float32", "uint32"), ("int64", "uint64"),
                                         ("uint32", "uint64"), ("float64", "uint32")])
def test_keyvalue_select_unaligned(xss, cuda, ktype, vtype, pad):
    x = get_array("random", ktype, N, 21 + pad)
    v = np.arange(N, dtype=vtype)
    for k in _ks(N):
        kb, kp = _dev(cuda, x, pad)
        vb, vp = _dev(cuda, v, (pad * 3) % 4)
        xss.gpu_keyvalue_select(ktype, vtype, kp, vp, k, N, False, False)
        xss.stream_status()
        gk = _back(kb, x, pad)
        gv = _back(vb, v, (pad * 3) % 4)
        what = f"kvselect {ktype}/{vtype} pad={pad} k={k}"
        assert_partitioned(gk, k, ref_sorted(x)[k], False, what)
        assert_pairs_preserved(x, v, gk, gv, what)


@pytest.mark.parametrize("pad", [0, 1])
@pytest.mark.parametrize("dtype", ["float32", "int64"])
def test_argselect_unaligned(xss, cuda, dtype, pad):
    torch = cuda
    x = get_array("random", dtype, N, 31 + pad)
    for k in _ks(N):
        buf, ptr = _dev(cuda, x, pad)
        arg = torch.zeros(N, dtype=torch.int64, device="cuda")
        xss.gpu_argselect(dtype, ptr, arg.data_ptr(), k, N, False)
        xss.stream_status()
        kept = _back(buf, x, pad)
        assert np.array_equal(kept.view(UINT[x.itemsize]), x.view(UINT[x.itemsize]))
        a = arg.cpu().numpy()
        what = f"argselect {dtype} pad={pad} k={k}"
        assert_is_permutation(a, N, what)
        assert_partitioned(x[a], k, ref_sorted(x)[k], False, what)

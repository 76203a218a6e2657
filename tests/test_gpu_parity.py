"""GPU parity against the CPU oracle and the reference's golden outputs.

Restates the reference's tests (tests/test-qsort.cpp, tests/test-keyvalue.cpp)
over the C ABI: every key type, every array shape, ascending and descending,
sizes that cross the one-CTA path, tile boundaries and the multi-tile radix
path.  Sorted keys must equal the oracle's byte for byte after canonicalising
+-0 and NaN payloads; argsort/argselect must return permutations whose gathered
keys match; select must put the exact k-th element at k with the partition
property; key-value results must keep every (key, value) pair.
"""
import ctypes

import numpy as np
import pytest

from golden_io import DT, check_case, load as load_golden
from xss_arrays import (EXTRA_SHAPES, KEY_TYPES, KV_TYPES, QNAN_BITS, SHAPES, UINT,
                        assert_arg_sorted, assert_pairs_preserved, assert_partitioned,
                        assert_same_sorted, get_array, is_nan_test, kv_values, ref_sorted)

pytestmark = pytest.mark.gpu

ALL_SHAPES = SHAPES + EXTRA_SHAPES
SIZES_SORT = [0, 1, 2, 3, 5, 8, 16, 17, 31, 32, 33, 64, 100, 127, 128, 129, 255, 256, 257, 511,
              512, 513, 1000, 1023, 1024, 2047, 2048, 4095, 4096, 4097, 5000, 8192, 12345,
              65537, 100_000]
SIZES_SEL = [0, 1, 2, 3, 5, 17, 100, 513, 1023, 4096, 4097, 6000, 50_000, 200_001]


def hasnan_for(shape):
    return is_nan_test(shape) or shape == "mixed_special"


def _k_values(n, rng):
    if n == 0:
        return [0]
    ks = {0, n - 1, n // 2, (2 * n) // 3, int(rng.integers(0, n))}
    return sorted(ks)


@pytest.mark.parametrize("dtype", KEY_TYPES)
def test_qsort_matches_oracle(xss, oracle, cuda, dtype):
    for shape in ALL_SHAPES:
        hn = hasnan_for(shape)
        for n in SIZES_SORT:
            x = get_array(shape, dtype, n, seed=n + 1)
            for desc in (False, True):
                got = x.copy()
                xss.qsort(got, hn, desc)
                want = x.copy()
                assert oracle.qsort(DT[dtype], want.ctypes.data, n, int(hn), int(desc)) == 0
                what = f"qsort {dtype} {shape} n={n} desc={desc}"
                assert_same_sorted(got, want, what)
                if hn and x.dtype.kind == "f" and n > 1:
                    nan = np.isnan(got)
                    cnt = int(nan.sum())
                    if cnt:
                        # canonical quiet NaN in the NaN slots, at the end (asc) or front (desc)
                        assert (got.view(UINT[got.itemsize])[nan] == QNAN_BITS[got.itemsize]).all(), what
                        assert nan[:cnt].all() if desc else nan[-cnt:].all(), what


@pytest.mark.parametrize("dtype", KEY_TYPES)
def test_argsort_matches_oracle(xss, oracle, cuda, dtype):
    for shape in ALL_SHAPES:
        hn = hasnan_for(shape)
        for n in SIZES_SORT[::2] + [4097, 65537]:
            x = get_array(shape, dtype, n, seed=n + 2)
            for desc in (False, True):
                keep = x.copy()
                arg = xss.argsort(x, hn, desc)
                assert np.array_equal(x.view(UINT[x.itemsize]), keep.view(UINT[x.itemsize]))
                want = x.copy()
                assert oracle.qsort(DT[dtype], want.ctypes.data, n, int(hn), int(desc)) == 0
                assert_arg_sorted(x, arg, want, f"argsort {dtype} {shape} n={n} desc={desc}")


@pytest.mark.parametrize("dtype", KEY_TYPES)
def test_qselect_and_partial_qsort(xss, oracle, cuda, dtype):
    rng = np.random.default_rng(5)
    for shape in ALL_SHAPES:
        hn = hasnan_for(shape)
        for n in SIZES_SEL:
            x = get_array(shape, dtype, n, seed=n + 3)
            srt = {d: ref_sorted(x, d) for d in (False, True)}
            for k in _k_values(n, rng):
                for desc in (False, True):
                    what = f"{dtype} {shape} n={n} k={k} desc={desc}"
                    got = x.copy()
                    xss.qselect(got, k, hn, desc)
                    if n > 1:
                        assert_partitioned(got, k, srt[desc][k], desc, "qselect " + what)
                        assert_same_sorted(ref_sorted(got), srt[False], "qselect multiset " + what)
                    got = x.copy()
                    kk = min(n, k + 1)
                    xss.partial_qsort(got, kk, hn, desc)
                    if n > 1:
                        assert_same_sorted(got[:kk], srt[desc][:kk], "partial " + what)
                        assert_same_sorted(ref_sorted(got), srt[False], "partial multiset " + what)
                        if kk < n:
                            assert_partitioned(got, kk - 1, srt[desc][kk - 1], desc,
                                               "partial tail " + what)


@pytest.mark.parametrize("dtype", KEY_TYPES)
def test_argselect(xss, oracle, cuda, dtype):
    rng = np.random.default_rng(6)
    for shape in ALL_SHAPES:
        hn = hasnan_for(shape)
        for n in SIZES_SEL:
            x = get_array(shape, dtype, n, seed=n + 4)
            srt = ref_sorted(x)
            for k in _k_values(n, rng):
                if n == 0:
                    continue
                arg = xss.argselect(x, k, hn)
                what = f"argselect {dtype} {shape} n={n} k={k}"
                from xss_arrays import assert_is_permutation
                assert_is_permutation(arg, n, what)
                if n > 1:
                    assert_partitioned(x[arg.astype(np.int64)], k, srt[k], False, what)


@pytest.mark.parametrize("ktype", KV_TYPES)
def test_keyvalue_family(xss, oracle, cuda, ktype):
    rng = np.random.default_rng(7)
    for vtype in KV_TYPES:
        for shape in ALL_SHAPES:
            hn = hasnan_for(shape)
            for n in [0, 1, 2, 33, 1000, 4096, 4097, 30_000, 100_001]:
                x = get_array(shape, ktype, n, seed=n + 5)
                v = kv_values(vtype, n, seed=n)
                for desc in (False, True):
                    what = f"kv {ktype}/{vtype} {shape} n={n} desc={desc}"
                    k, w = x.copy(), v.copy()
                    xss.keyvalue_qsort(k, w, hn, desc)
                    ok, ow = x.copy(), v.copy()
                    assert oracle.keyvalue_qsort(DT[ktype], DT[vtype], ok.ctypes.data,
                                                 ow.ctypes.data, n, int(hn), int(desc)) == 0
                    assert_same_sorted(k, ok, what)
                    assert_pairs_preserved(x, v, k, w, what)
                    if n < 2:
                        continue
                    kk = int(rng.integers(0, n))
                    k, w = x.copy(), v.copy()
                    xss.keyvalue_select(k, w, kk, hn, desc)
                    assert_partitioned(k, kk, ok[kk], desc, "kvselect " + what)
                    assert_pairs_preserved(x, v, k, w, "kvselect " + what)
                    k, w = x.copy(), v.copy()
                    xss.keyvalue_partial_sort(k, w, kk + 1, hn, desc)
                    assert_same_sorted(k[:kk + 1], ok[:kk + 1], "kvpartial " + what)
                    assert_pairs_preserved(x, v, k, w, "kvpartial " + what)


@pytest.mark.parametrize("ktype", KEY_TYPES)
def test_keyvalue_16bit_payloads(xss, oracle, cuda, ktype):
    """uint16 / int16 / _Float16 values (beyond the reference's 32/64-bit
    values): every key type, sort / select / partial sort.  Passes carrying
    values are stable, so a sort's values must be exactly the input values in
    the stable order of the keys' codes."""
    from xss_arrays import bit_code
    rng = np.random.default_rng(8)
    for vtype in ("uint16", "int16", "float16"):
        for shape in ("random", "smallrange", "reverse", "mixed_special", "rand_with_nan"):
            hn = hasnan_for(shape)
            for n in [0, 1, 2, 33, 1000, 4096, 4097, 30_000, 100_001]:
                x = get_array(shape, ktype, n, seed=n + 9)
                v = kv_values(vtype, n, seed=n)
                for desc in (False, True):
                    what = f"kv {ktype}/{vtype} {shape} n={n} desc={desc}"
                    k, w = x.copy(), v.copy()
                    xss.keyvalue_qsort(k, w, hn, desc)
                    ok, ow = x.copy(), v.copy()
                    assert oracle.keyvalue_qsort(DT[ktype], DT[vtype], ok.ctypes.data,
                                                 ow.ctypes.data, n, int(hn), int(desc)) == 0
                    assert_same_sorted(k, ok, what)
                    stable = np.argsort(bit_code(x, desc), kind="stable")
                    assert np.array_equal(w.view(np.uint16), v[stable].view(np.uint16)), what
                    if n < 2:
                        continue
                    kk = int(rng.integers(0, n))
                    k, w = x.copy(), v.copy()
                    xss.keyvalue_select(k, w, kk, hn, desc)
                    assert_partitioned(k, kk, ok[kk], desc, "kvselect " + what)
                    assert_pairs_preserved(x, v, k, w, "kvselect " + what)
                    k, w = x.copy(), v.copy()
                    xss.keyvalue_partial_sort(k, w, kk + 1, hn, desc)
                    assert_same_sorted(k[:kk + 1], ok[:kk + 1], "kvpartial " + what)
                    assert_pairs_preserved(x, v, k, w, "kvpartial " + what)


class _HostApi:
    """The library's xss_* host entry points under the oracle's names."""

    def __init__(self, L):
        for name in ("qsort", "qselect", "partial_qsort", "argsort", "argselect",
                     "keyvalue_qsort", "keyvalue_select", "keyvalue_partial_sort"):
            setattr(self, name, getattr(L, "xss_" + name))


def test_golden_fixtures(xss, cuda):
    """Outputs of the reference library itself (tests/golden/make_golden.py)."""
    cases, get = load_golden()
    api = _HostApi(xss.lib())
    for cid, c in cases.items():
        check_case(api, c, get, cid)


def test_reference_c_symbols(xss, cuda):
    """keyvalue_qsort_<k>_<v> (lib/x86simdsort.cpp:298-339): ascending, hasnan."""
    L = xss.lib()
    for kname, kt in (("float", "float32"), ("uint64", "uint64"), ("int32", "int32"),
                      ("uint32", "uint32")):
        for vname, vt in (("uint32", "uint32"), ("uint64", "uint64")):
            x = get_array("rand_with_nan" if kt == "float32" else "random", kt, 9000, 3)
            v = np.arange(9000, dtype=vt)
            k, w = x.copy(), v.copy()
            getattr(L, f"keyvalue_qsort_{kname}_{vname}")(ctypes.c_void_p(k.ctypes.data),
                                                           ctypes.c_void_p(w.ctypes.data),
                                                           ctypes.c_size_t(9000))
            assert_same_sorted(k, ref_sorted(x), kname + vname)
            assert_same_sorted(k, x[w.astype(np.int64)], kname + vname + " gather")


def test_device_pointer_api_with_caller_workspace(xss, cuda):
    torch = cuda
    stream = torch.cuda.Stream()
    for dtype in ("float32", "int64", "float16", "uint32"):
        n = 300_000
        x = get_array("mixed_special" if dtype.startswith("f") else "random", dtype, n, 8)
        d = torch.from_numpy(x.view(np.uint8).copy()).cuda()
        ws_bytes = xss.workspace_size("qsort", dtype, n)
        ws = torch.empty(ws_bytes, dtype=torch.uint8, device="cuda")
        with torch.cuda.stream(stream):
            xss.gpu_qsort(dtype, d.data_ptr(), n, True, False, ws.data_ptr(), ws_bytes,
                          stream.cuda_stream)
        xss.stream_status(stream.cuda_stream)
        got = d.cpu().numpy().view(x.dtype)
        assert_same_sorted(got, ref_sorted(x), "device " + dtype)
        # too-small caller workspace is refused, not overrun
        with pytest.raises(xss.XssError) as e:
            xss.gpu_qsort(dtype, d.data_ptr(), n, True, False, ws.data_ptr(), ws_bytes - 256,
                          stream.cuda_stream)
        assert e.value.code == 2

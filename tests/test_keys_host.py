"""Exhaustive / sampled checks of the order-preserving key transform on the host.

The transform (x86-simd-sort_gb300/csrc/xss_keys.cuh) is what makes a radix
sort reproduce the reference comparator's order (utils/custom-compare.h:11-34):
it must be a bijection, invert exactly, order numbers like the comparator,
put every NaN after +inf (before it when descending) and keep NaN payloads
unless canonicalisation is asked for.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from xss_arrays import UINT, get_array, order_code

HERE = os.path.dirname(os.path.abspath(__file__))
SO = os.path.join(HERE, "_build", "libkeys_host.so")
KIND = {"u": 0, "i": 1, "f": 2}


@pytest.fixture(scope="module")
def kh():
    src = os.path.join(HERE, "keys_host.cu")
    hdr = os.path.join(os.path.dirname(HERE), "x86-simd-sort_gb300", "csrc", "xss_keys.cuh")
    if not os.path.exists(SO) or os.path.getmtime(SO) < max(os.path.getmtime(src),
                                                            os.path.getmtime(hdr)):
        os.makedirs(os.path.dirname(SO), exist_ok=True)
        nvcc = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
        subprocess.run([nvcc, "-shared", "-Xcompiler", "-fPIC", "-std=c++17", "-o", SO, src],
                       check=True)
    return ctypes.CDLL(SO)


def _fwd(kh, x, kind, desc, canon=0):
    out = np.empty_like(x)
    getattr(kh, f"kh_to_code{8 * x.itemsize}")(ctypes.c_void_p(x.ctypes.data),
                                               ctypes.c_void_p(out.ctypes.data),
                                               ctypes.c_size_t(x.size), kind, desc, canon)
    return out


def _inv(kh, c, kind, desc):
    out = np.empty_like(c)
    getattr(kh, f"kh_from_code{8 * c.itemsize}")(ctypes.c_void_p(c.ctypes.data),
                                                 ctypes.c_void_p(out.ctypes.data),
                                                 ctypes.c_size_t(c.size), kind, desc)
    return out


def _check(kh, vals: np.ndarray, desc: int):
    bits = np.ascontiguousarray(vals).view(UINT[vals.itemsize])
    kind = KIND[vals.dtype.kind]
    codes = _fwd(kh, bits, kind, desc)
    assert np.array_equal(_inv(kh, codes, kind, desc), bits), "inverse"
    assert np.unique(codes).size == np.unique(bits).size, "bijection"
    # code order refines the comparator order (ties only between values it calls equal)
    oc = order_code(vals, bool(desc))
    o = oc[np.argsort(codes, kind="stable")]
    assert (o[1:] >= o[:-1]).all(), "order"
    if vals.dtype.kind == "f":
        nan = np.isnan(vals)
        fin = ~nan
        if nan.any() and fin.any():
            if desc:
                assert codes[nan].max() < codes[fin].min()
            else:
                assert codes[nan].min() > codes[fin].max()
        zero = vals == 0
        neg0 = zero & (bits >> (8 * vals.itemsize - 1)).astype(bool)
        if neg0.any() and (zero & ~neg0).any():
            # -0 and +0 adjacent, -0 first in ascending order
            assert abs(int(codes[neg0][0]) - int(codes[zero & ~neg0][0])) == 1


@pytest.mark.parametrize("dtype", ["uint16", "int16", "float16"])
@pytest.mark.parametrize("desc", [0, 1])
def test_all_16bit_patterns(kh, dtype, desc):
    vals = np.arange(1 << 16, dtype=np.uint16).view(np.dtype(dtype))
    _check(kh, vals, desc)


@pytest.mark.parametrize("dtype", ["uint32", "int32", "float32", "uint64", "int64", "float64"])
@pytest.mark.parametrize("desc", [0, 1])
def test_sampled_wide_patterns(kh, dtype, desc):
    dt = np.dtype(dtype)
    rng = np.random.default_rng(11)
    raw = rng.integers(0, np.iinfo(UINT[dt.itemsize]).max, 200_000, dtype=UINT[dt.itemsize],
                       endpoint=True)
    specials = get_array("mixed_special", dt, 5000, 3).view(UINT[dt.itemsize])
    edges = np.array([0, 1, (1 << (8 * dt.itemsize - 1)) - 1, 1 << (8 * dt.itemsize - 1),
                      (1 << (8 * dt.itemsize)) - 1], dtype=np.uint64).astype(UINT[dt.itemsize])
    vals = np.unique(np.concatenate([raw, specials, edges])).view(dt)
    _check(kh, vals, desc)


@pytest.mark.parametrize("dtype", ["float16", "float32", "float64"])
def test_canonical_nan(kh, dtype):
    dt = np.dtype(dtype)
    x = get_array("mixed_special", dt, 4000, 9)
    bits = x.view(UINT[dt.itemsize])
    nan = np.isnan(x)
    assert nan.sum() > 10
    codes = _fwd(kh, bits, 2, 0, canon=1)
    assert np.unique(codes[nan]).size == 1
    back = _inv(kh, codes, 2, 0)
    qn = {2: 0x7C01, 4: 0x7FC00000, 8: 0x7FF8000000000000}[dt.itemsize]
    assert (back[nan] == qn).all()
    assert np.array_equal(back[~nan], bits[~nan])


@pytest.mark.parametrize("bits", [16, 32, 64])
def test_branch_free_codec_matches_transform(kh, bits):
    """The passes' branch-free codec equals to_code / from_code on every 16-bit
    pattern and on sampled 32/64-bit patterns plus the edge values (zeros,
    infinities, the NaN range ends), for every kind, order and NaN rule."""
    ut = {16: np.uint16, 32: np.uint32, 64: np.uint64}[bits]
    if bits == 16:
        x = np.arange(1 << 16, dtype=np.uint16)
    else:
        rng = np.random.default_rng(bits)
        x = rng.integers(0, np.iinfo(ut).max, 1 << 20, dtype=ut, endpoint=True)
        sign = ut(1) << ut(bits - 1)
        exp = {32: 0x7f800000, 64: 0x7ff0000000000000}[bits]
        edges = [0, 1, exp, exp + 1, exp | (exp >> 9), sign - 1, sign, sign | exp,
                 sign | (exp + 1), np.iinfo(ut).max, np.iinfo(ut).max - 1]
        x = np.concatenate([x, np.array(edges, dtype=ut)])
    f = getattr(kh, f"kh_codec{bits}")
    f.restype = ctypes.c_size_t
    for kind in (0, 1, 2):
        for desc in (0, 1):
            for canon in (0, 1):
                bad = f(ctypes.c_void_p(x.ctypes.data), ctypes.c_size_t(x.size), kind, desc,
                        canon)
                assert bad == 0, (bits, kind, desc, canon, bad)


@pytest.mark.parametrize("dtype", ["float16", "int16", "uint16"])
def test_bit_code_helper_is_the_library_code(kh, dtype):
    """The tests' bit_code (exact stable-order checks) equals to_code on every
    16-bit pattern, ascending and descending."""
    from xss_arrays import bit_code
    x = np.arange(1 << 16, dtype=np.uint16).view(dtype)
    for desc in (0, 1):
        got = _fwd(kh, x.view(np.uint16), KIND[np.dtype(dtype).kind], desc)
        assert np.array_equal(got.astype(np.uint64), bit_code(x, bool(desc)))

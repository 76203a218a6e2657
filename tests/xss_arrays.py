"""Seeded input generators and property checkers for the parity tests.

Generators restate the reference's array shapes (utils/rand_array.h:66-169)
with fixed seeds (the reference seeds from std::random_device,
tests/test-qsort-common.h:4).  Checkers restate tests/test-qsort-common.h:11-119
and tests/test-keyvalue.cpp:44-171: byte equality of sorted keys after
canonicalising what the reference's comparator treats as equal (-0.0 / +0.0,
NaN payloads), permutation validity for argsort, the partition property for
select, and (key, value) multiset preservation for the key-value family.
"""
from __future__ import annotations

import numpy as np

SHAPES = ["random", "constant", "sorted", "reverse", "smallrange", "max_at_the_end",
          "random_5d", "rand_max", "rand_with_nan", "rand_with_max_and_nan"]
# extra shape of this suite: negative values, +-0, +-inf, subnormals and NaNs
# with random payloads and both signs (key-value / arg paths keep payloads)
EXTRA_SHAPES = ["mixed_special"]

KEY_TYPES = ["uint16", "int16", "float16", "float32", "float64", "uint32", "int32",
             "uint64", "int64"]
KV_TYPES = ["uint32", "int32", "float32", "uint64", "int64", "float64"]
UINT = {2: np.uint16, 4: np.uint32, 8: np.uint64}
SIGN = {2: 0x8000, 4: 0x80000000, 8: 0x8000000000000000}
NEG_NANS = {2: 0x3FF, 4: 0x7FFFFF, 8: 0xFFFFFFFFFFFFF}
# quiet NaN the reference writes (xss-custom-float.h:81-85 for _Float16)
QNAN_BITS = {2: 0x7C01, 4: 0x7FC00000, 8: 0x7FF8000000000000}


def is_nan_test(shape: str) -> bool:
    return "nan" in shape


def _qnan(dt: np.dtype):
    return np.array([QNAN_BITS[dt.itemsize]], dtype=UINT[dt.itemsize]).view(dt)[0]


def _uniform(rng, dt: np.dtype, n: int, lo=None, hi=None) -> np.ndarray:
    if dt.kind == "f":
        if dt == np.float16 and lo is None:
            # (float)rand()/RAND_MAX for _Float16 (rand_array.h:31-40)
            return rng.random(n).astype(np.float16)
        info = np.finfo(dt)
        lo = float(info.tiny) if lo is None else lo
        hi = float(info.max) if hi is None else hi
        return (lo + (rng.random(n) * (hi / 2 - lo / 2)) * 2).astype(dt)
    info = np.iinfo(dt)
    lo = int(info.min) if lo is None else lo
    hi = int(info.max) if hi is None else hi
    return rng.integers(lo, hi, n, dtype=dt, endpoint=True)


def get_array(shape: str, dtype, n: int, seed: int = 0) -> np.ndarray:
    dt = np.dtype(dtype)
    rng = np.random.default_rng([seed, n, SHAPES.index(shape) if shape in SHAPES else 99,
                                 dt.num])
    if n == 0:
        return np.zeros(0, dtype=dt)
    isf = dt.kind == "f"
    top = np.array(np.inf, dtype=dt) if isf else np.iinfo(dt).max
    if shape == "random":
        return _uniform(rng, dt, n)
    if shape == "sorted":
        return np.sort(_uniform(rng, dt, n))
    if shape == "reverse":
        return np.sort(_uniform(rng, dt, n))[::-1].copy()
    if shape == "constant":
        return np.full(n, _uniform(rng, dt, 1)[0], dtype=dt)
    if shape == "smallrange":
        return _uniform(rng, dt, n, 1, 20)
    if shape == "random_5d":
        half = max(1, int(0.5 * n))
        a = np.zeros(n, dtype=dt)
        a[:half] = _uniform(rng, dt, half)
        rng.shuffle(a)
        return a
    if shape == "max_at_the_end":
        a = _uniform(rng, dt, n)
        a[-1] = top
        return a
    if shape == "rand_with_nan":
        a = _uniform(rng, dt, n)
        idx = rng.integers(0, n, 10 % n)
        a[idx] = _qnan(dt) if isf else top
        return a
    if shape == "rand_max":
        a = _uniform(rng, dt, n)
        a[rng.random(n) < 0.5] = top
        return a
    if shape == "rand_with_max_and_nan":
        a = _uniform(rng, dt, n)
        r = rng.integers(0, 4, n)
        a[r == 2] = top
        a[r == 3] = _qnan(dt) if isf else top
        return a
    if shape == "mixed_special":
        if not isf:
            return _uniform(rng, dt, n)
        a = (rng.standard_normal(n) * 100).astype(dt)
        r = rng.integers(0, 16, n)
        a[r == 0] = 0.0
        a[r == 1] = -0.0
        a[r == 2] = np.inf
        a[r == 3] = -np.inf
        u = a.view(UINT[dt.itemsize])
        nanpos = np.nonzero(r == 4)[0]
        if nanpos.size:
            mant = rng.integers(1, NEG_NANS[dt.itemsize], nanpos.size, endpoint=True,
                                dtype=np.uint64).astype(UINT[dt.itemsize])
            expo = np.array(_exp_bits(dt.itemsize), dtype=UINT[dt.itemsize])
            sign = rng.integers(0, 2, nanpos.size).astype(UINT[dt.itemsize]) * \
                UINT[dt.itemsize](SIGN[dt.itemsize])
            u[nanpos] = sign | expo | mant
        sub = np.nonzero(r == 5)[0]
        if sub.size:
            u[sub] = rng.integers(1, NEG_NANS[dt.itemsize] // 2, sub.size,
                                  dtype=np.uint64).astype(UINT[dt.itemsize])
        return a
    raise ValueError(shape)


def _exp_bits(nbytes: int) -> int:
    return {2: 0x7C00, 4: 0x7F800000, 8: 0x7FF0000000000000}[nbytes]


def kv_values(dtype, n: int, seed: int = 1) -> np.ndarray:
    """Distinct-ish payloads so value mix-ups are visible."""
    dt = np.dtype(dtype)
    rng = np.random.default_rng([seed, n, dt.num, 7])
    if dt.kind == "f":
        return rng.standard_normal(n).astype(dt)
    return rng.integers(0, np.iinfo(dt).max, n, dtype=dt, endpoint=True)


# ---- canonical forms ------------------------------------------------------------
def canon(a: np.ndarray) -> np.ndarray:
    """Bit patterns with every NaN made one pattern and -0.0 made +0.0."""
    a = np.ascontiguousarray(a)
    u = a.view(UINT[a.itemsize]).copy()
    if a.dtype.kind == "f":
        u[np.isnan(a)] = QNAN_BITS[a.itemsize]
        u[a == 0] = 0
    return u


def order_code(a: np.ndarray, descending: bool = False) -> np.ndarray:
    """Unsigned codes whose order is the reference comparator's order, with
    values it treats as equal mapped to equal codes (uint64 for all widths)."""
    nb = a.itemsize
    u = canon(a).astype(np.uint64)
    sign = np.uint64(SIGN[nb])
    full = np.uint64((1 << (8 * nb)) - 1)
    if a.dtype.kind == "f":
        neg = (u & sign) != 0
        c = np.where(neg, (~u) & full, u | sign)
        c = np.where(np.isnan(a), full, c)
    elif a.dtype.kind == "i":
        c = u ^ sign
    else:
        c = u
    return ((~c) & full) if descending else c


def bit_code(a: np.ndarray, descending: bool = False) -> np.ndarray:
    """The library's own sort code of every bit pattern (uint64 for all widths):
    like order_code but -0.0 before +0.0 and NaNs ordered by their bits (all
    after +inf), so a stable sort by it is the exact order the library's
    stable paths (key-value, argsort) produce."""
    nb = a.itemsize
    u = np.ascontiguousarray(a).view(UINT[nb]).astype(np.uint64)
    sign = np.uint64(SIGN[nb])
    full = np.uint64((1 << (8 * nb)) - 1)
    if a.dtype.kind == "f":
        neg = (u & sign) != 0
        c = np.where(neg, (~u) & full, u | sign)
        c = (c - np.uint64(NEG_NANS[nb])) & full
    elif a.dtype.kind == "i":
        c = u ^ sign
    else:
        c = u
    return ((~c) & full) if descending else c


# ---- checkers -------------------------------------------------------------------
def assert_same_sorted(got: np.ndarray, want: np.ndarray, what: str = "") -> None:
    g, w = canon(got), canon(want)
    if not np.array_equal(g, w):
        bad = np.nonzero(g != w)[0]
        raise AssertionError(f"{what}: {bad.size} positions differ, first at {bad[:5]}: "
                             f"got {got[bad[:5]]} want {want[bad[:5]]}")


def assert_is_permutation(arg: np.ndarray, n: int, what: str = "") -> None:
    assert arg.size == n, f"{what}: {arg.size} indices for {n} elements"
    if n:
        assert np.array_equal(np.sort(arg.astype(np.uint64)), np.arange(n, dtype=np.uint64)), \
            f"{what}: indices are not a permutation"


def assert_arg_sorted(arr: np.ndarray, arg: np.ndarray, sorted_ref: np.ndarray,
                      what: str = "") -> None:
    assert_is_permutation(arg, arr.size, what)
    assert_same_sorted(arr[arg.astype(np.int64)], sorted_ref, what)


def assert_partitioned(arr: np.ndarray, k: int, kth, descending: bool, what: str = "") -> None:
    c = order_code(arr, descending)
    ck = order_code(np.array([kth], dtype=arr.dtype), descending)[0]
    assert c[k] == ck, f"{what}: kth element {arr[k]} != {kth}"
    if k > 0:
        assert c[:k].max() <= ck, f"{what}: left partition has a larger element"
    if k + 1 < arr.size:
        assert c[k + 1:].min() >= ck, f"{what}: right partition has a smaller element"


def assert_pairs_preserved(k_in, v_in, k_out, v_out, what: str = "") -> None:
    a = np.lexsort((canon(v_in), canon(k_in)))
    b = np.lexsort((canon(v_out), canon(k_out)))
    assert np.array_equal(canon(k_in)[a], canon(k_out)[b]) and \
        np.array_equal(canon(v_in)[a], canon(v_out)[b]), f"{what}: (key, value) pairs changed"


def ref_sorted(arr: np.ndarray, descending: bool = False) -> np.ndarray:
    """Sorted copy in the reference comparator's order (ties arbitrary)."""
    order = np.argsort(order_code(arr, descending), kind="stable")
    return arr[order]

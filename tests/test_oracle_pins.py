"""Pins the CPU oracle (test infrastructure) before it is trusted as a checker.

1. the reference's comparator known-answer table (tests/test-qsort.cpp:261-292);
2. the golden fixtures produced by the reference library itself
   (tests/golden/make_golden.py);
3. the live reference built from source in oracle/_ref, where the host can
   build it (skipped elsewhere).
"""
import ctypes

import numpy as np
import pytest

from golden_io import check_case as _check_case
from golden_io import load as load_golden
from xss_arrays import (SHAPES, EXTRA_SHAPES, assert_arg_sorted, assert_pairs_preserved,
                        assert_partitioned, assert_same_sorted, canon, get_array,
                        is_nan_test, kv_values, ref_sorted)

DT = {"uint16": 0, "int16": 1, "float16": 2, "uint32": 3, "int32": 4, "float32": 5,
      "uint64": 6, "int64": 7, "float64": 8}

# (op, a, b, expected) for a, b in {nan, inf}; op: 0 <, 1 <=, 2 >, 3 >=, 4 ==
COMPARATOR_KAT = [
    (0, "nan", "inf", False), (0, "nan", "nan", False), (0, "inf", "nan", True),
    (0, "inf", "inf", False),
    (1, "nan", "inf", False), (1, "nan", "nan", True), (1, "inf", "nan", True),
    (1, "inf", "inf", True),
    (3, "nan", "inf", True), (3, "nan", "nan", True), (3, "inf", "nan", False),
    (3, "inf", "inf", True),
    (2, "nan", "inf", True), (2, "nan", "nan", False), (2, "inf", "nan", False),
    (2, "inf", "inf", False),
    (4, "nan", "inf", False), (4, "nan", "nan", True), (4, "inf", "nan", False),
    (4, "inf", "inf", True),
]


@pytest.mark.parametrize("dtype", ["float16", "float32", "float64"])
def test_comparator_known_answers(oracle, dtype):
    dt = np.dtype(dtype)
    vals = {"nan": np.array([np.nan], dt), "inf": np.array([np.inf], dt)}
    if dt == np.float16:
        vals["nan"] = np.array([0x7C01], np.uint16).view(dt)  # the reference's _Float16 qNaN
    for op, a, b, want in COMPARATOR_KAT:
        got = oracle.compare(DT[dtype], op, vals[a].ctypes.data, vals[b].ctypes.data)
        assert got == int(want), (dtype, op, a, b)


def test_oracle_matches_golden(oracle):
    cases, get = load_golden()
    assert len(cases) > 3000
    for cid, c in cases.items():
        _check_case(oracle, c, get, cid)


def test_golden_outputs_are_sorted():
    """The fixtures themselves satisfy the sort contract (guards a bad regeneration)."""
    cases, get = load_golden()
    for cid, c in cases.items():
        if c["op"] == "qsort":
            x, y = get(f"{cid}_in"), get(f"{cid}_out")
            assert_same_sorted(y, ref_sorted(x, c["desc"]), f"case {cid}")


def test_qsort_nan_slots_hold_quiet_nan_in_golden():
    """The reference writes the canonical quiet NaN into NaN slots for qsort with hasnan
    (src/xss-common-qsort.h:107-135): last slots ascending, first slots descending."""
    cases, get = load_golden()
    qn = {"float16": 0x7C01, "float32": 0x7FC00000, "float64": 0x7FF8000000000000}
    seen = 0
    for cid, c in cases.items():
        if c["op"] != "qsort" or not c["hasnan"] or c["dtype"] not in qn or c["n"] < 2:
            continue
        y = get(f"{cid}_out")
        nan = np.isnan(y)
        if not nan.any():
            continue
        u = y.view({2: np.uint16, 4: np.uint32, 8: np.uint64}[y.itemsize])
        assert (u[nan] == qn[c["dtype"]]).all()
        cnt = int(nan.sum())
        assert nan[:cnt].all() if c["desc"] else nan[-cnt:].all()
        seen += 1
    assert seen > 20


def test_oracle_matches_live_reference(oracle):
    from oracle import pyoracle
    ref = pyoracle.reference()
    if ref is None:
        pytest.skip("reference library not built on this host (needs x86-64 sources)")
    for dtype in DT:
        for shape in SHAPES + EXTRA_SHAPES:
            for n in (3, 64, 777, 3000):
                hasnan = int(is_nan_test(shape) or shape == "mixed_special")
                x = get_array(shape, dtype, n, seed=77)
                for desc in (0, 1):
                    a, b = x.copy(), x.copy()
                    assert ref.qsort(DT[dtype], a.ctypes.data, n, hasnan, desc) == 0
                    assert oracle.qsort(DT[dtype], b.ctypes.data, n, hasnan, desc) == 0
                    assert_same_sorted(a, b, f"{dtype} {shape} {n} {desc}")
                if np.dtype(dtype).itemsize >= 4:
                    v = kv_values("uint64", n)
                    a, b, va, vb = x.copy(), x.copy(), v.copy(), v.copy()
                    assert ref.keyvalue_qsort(DT[dtype], 6, a.ctypes.data, va.ctypes.data, n,
                                              hasnan, 1) == 0
                    assert oracle.keyvalue_qsort(DT[dtype], 6, b.ctypes.data, vb.ctypes.data, n,
                                                 hasnan, 1) == 0
                    assert_same_sorted(a, b, f"kv {dtype} {shape} {n}")
                    assert_pairs_preserved(x, v, a, va, "ref")
                    assert_pairs_preserved(x, v, b, vb, "oracle")


def test_parallel_oracle_matches_scalar(oracle):
    """The task-parallel CPU baseline gives the scalar oracle's result."""
    for dtype in ("float32", "int64", "float64", "uint16"):
        x = get_array("mixed_special" if dtype.startswith("f") else "random", dtype, 300_000, 5)
        a, b = x.copy(), x.copy()
        assert oracle.qsort_mt(DT[dtype], a.ctypes.data, a.size, 1, 0, 4) == 0
        assert oracle.qsort(DT[dtype], b.ctypes.data, b.size, 1, 0) == 0
        assert_same_sorted(a, b, dtype)
        arg = np.zeros(x.size, np.uint64)
        assert oracle.argsort_mt(DT[dtype], x.ctypes.data, arg.ctypes.data, x.size, 1, 1, 4) == 0
        assert_arg_sorted(x, arg, ref_sorted(x, True), dtype)
    k = get_array("random", "int64", 200_000, 6)
    v = np.arange(k.size, dtype=np.uint64)
    a, va = k.copy(), v.copy()
    assert oracle.keyvalue_qsort_mt(7, 6, a.ctypes.data, va.ctypes.data, a.size, 0, 0, 4) == 0
    assert_same_sorted(a, ref_sorted(k), "kv mt")
    assert_pairs_preserved(k, v, a, va, "kv mt")

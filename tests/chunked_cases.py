"""Parity cases of the chunked sort (arrays above one radix sort's size: sorted
in chunks, then merged), run with a small chunk length so that arrays of
thousands of keys take that path: ``XSS_MERGE_CHUNK=8192 python
tests/chunked_cases.py`` (test_gpu_chunked.py runs it so).  Every case is
checked against the CPU oracle; the merge is stable, so argsort and key-value
outputs must equal the stable order by the comparator's code exactly.
Prints one line per failure and exits non-zero if any.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
for p in (HERE, ROOT, os.path.join(ROOT, "x86-simd-sort_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

from golden_io import DT  # noqa: E402
from xss_arrays import (KEY_TYPES, KV_TYPES, assert_partitioned, assert_same_sorted,  # noqa: E402
                        bit_code, get_array, kv_values, ref_sorted)

SHAPES = ["random", "constant", "sorted", "reverse", "smallrange", "rand_with_nan",
          "mixed_special"]
SIZES = [8193, 20000, 65537, 100_000]


def main() -> int:
    import pyxss as xss
    from oracle import pyoracle
    orc = pyoracle.oracle()
    fails = []

    def check(cond, what):
        if not cond:
            fails.append(what)

    for dtype in KEY_TYPES:
        for shape in SHAPES:
            hn = shape in ("rand_with_nan", "mixed_special")
            for n in SIZES:
                x = get_array(shape, dtype, n, seed=n + 17)
                for desc in (False, True):
                    what = f"{dtype} {shape} n={n} desc={desc}"
                    got = x.copy()
                    xss.qsort(got, hn, desc)
                    want = x.copy()
                    assert orc.qsort(DT[dtype], want.ctypes.data, n, int(hn), int(desc)) == 0
                    try:
                        assert_same_sorted(got, want, "qsort " + what)
                    except AssertionError as e:
                        fails.append(str(e))
                    stable = np.argsort(bit_code(x, desc), kind="stable")
                    arg = xss.argsort(x, hn, desc)
                    check(np.array_equal(arg.astype(np.int64), stable), "argsort " + what)
                    if dtype in KV_TYPES and shape in ("random", "mixed_special", "smallrange"):
                        for vdt in ("uint32", "uint64"):
                            k, v = x.copy(), kv_values(vdt, n, seed=n)
                            v0 = v.copy()
                            xss.keyvalue_qsort(k, v, hn, desc)
                            check(np.array_equal(v, v0[stable]), f"kv {vdt} values " + what)
                            check(np.array_equal(k.view(np.uint8), x[stable].view(np.uint8)),
                                  f"kv {vdt} keys " + what)
                    if shape in ("random", "mixed_special") and n in (20000, 100_000):
                        srt = ref_sorted(x, desc)
                        for kth in (0, n // 3, n - 1):
                            got = x.copy()
                            xss.qselect(got, kth, hn, desc)
                            try:
                                assert_partitioned(got, kth, srt[kth], desc,
                                                   f"qselect k={kth} " + what)
                            except AssertionError as e:
                                fails.append(str(e))
                            if not desc:
                                a = xss.argselect(x, kth, hn)
                                try:
                                    assert_partitioned(x[a.astype(np.int64)], kth, srt[kth],
                                                       False, f"argselect k={kth} " + what)
                                except AssertionError as e:
                                    fails.append(str(e))
    for f in fails[:30]:
        print("FAIL", f)
    print(f"{len(fails)} failures")
    return 1 if fails else 0


if __name__ == "__main__":
    sys.exit(main())

"""Cases of the pipelined host-pointer sort with more chunks than the default
four, run in a child process whose chunk length is lowered through
XSS_MERGE_CHUNK (read once per process): ``XSS_MERGE_CHUNK=899840 python
tests/host_pipeline_cases.py`` cuts a 2^22 + 12345-key array into 5 chunks,
649984 into 7, 499968 into 9, so the merge levels that run between the chunk
sorts meet partial blocks at every level.  Host-pointer results must equal the
device-pointer sort of the same input exactly (both stable), and the float32
qsort the oracle's.  test_gpu_host_pipeline.py runs it.  Prints one line per
failure and exits non-zero if any.
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
from xss_arrays import assert_same_sorted, bit_code, get_array  # noqa: E402

N = (1 << 22) + 12345


def main() -> int:
    import torch
    import pyxss as xss
    from oracle import pyoracle
    orc = pyoracle.oracle()
    fails = []

    # key-value int64 -> uint64 with ties: the values' order among equal keys
    rng = np.random.default_rng(5)
    k = rng.integers(-2**40, 2**40, N, dtype=np.int64)
    k[::5] = -7
    v = np.arange(N, dtype=np.uint64)
    k_h, v_h = k.copy(), v.copy()
    xss.keyvalue_qsort(k_h, v_h, False, False)
    dk = torch.from_numpy(k.copy()).cuda()
    dv = torch.from_numpy(v.view(np.int64).copy()).cuda()
    xss.gpu_keyvalue_qsort("int64", "uint64", dk.data_ptr(), dv.data_ptr(), N, False, False)
    xss.stream_status()
    if not (np.array_equal(k_h, dk.cpu().numpy())
            and np.array_equal(v_h, dv.cpu().numpy().view(np.uint64))):
        fails.append("keyvalue int64->uint64")

    # float32 qsort with NaNs against the oracle
    x = get_array("rand_with_nan", "float32", N, seed=31)
    got = x.copy()
    xss.qsort(got, True, False)
    want = x.copy()
    try:
        assert orc.qsort(DT["float32"], want.ctypes.data, N, 1, 0) == 0
        assert_same_sorted(got, want, "qsort float32 rand_with_nan")
    except AssertionError as e:
        fails.append(f"qsort float32 rand_with_nan: {str(e)[:200]}")

    # argsort float64 (specials, descending): the stable order by the code
    y = get_array("mixed_special", "float64", N, seed=32)
    arg = xss.argsort(y, True, True)
    if not np.array_equal(arg.astype(np.int64), np.argsort(bit_code(y, True), kind="stable")):
        fails.append("argsort float64 mixed_special descending")

    for f in fails:
        print("FAIL", f)
    print(f"{len(fails)} failures (XSS_MERGE_CHUNK={os.environ.get('XSS_MERGE_CHUNK')})")
    return 1 if fails else 0


if __name__ == "__main__":
    sys.exit(main())

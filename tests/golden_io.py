"""Reader for tests/golden/golden.npz (written by tests/golden/make_golden.py)."""
import json
import os

import numpy as np

from xss_arrays import (assert_arg_sorted, assert_pairs_preserved, assert_partitioned,
                        assert_same_sorted)

DT = {"uint16": 0, "int16": 1, "float16": 2, "uint32": 3, "int32": 4, "float32": 5,
      "uint64": 6, "int64": 7, "float64": 8}

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "golden.npz")


def load():
    """Return (cases, get) where get(name) -> ndarray and cases maps id -> params."""
    z = np.load(PATH)
    blob = z["blob"]
    meta = json.loads(bytes(z["meta"]).decode())
    table = meta["arrays"]

    def get(name):
        off, nb, dt = table[name]
        return blob[off:off + nb].view(np.dtype(dt)).copy()

    return {int(k): v for k, v in meta["cases"].items()}, get


def check_case(fns, c, get, cid):
    """Run golden case `c` through `fns` and compare with the reference's output.

    `fns` exposes qsort, argsort, ... with the signatures of the C host entry
    points (dtype id, pointers, sizes, flags) -- the oracle, the reference shim
    and libxss_gb300's xss_* host functions all do."""
    op, n, desc, hasnan = c["op"], c["n"], int(c["desc"]), int(c["hasnan"])
    dtid = DT[c["dtype"]]
    x = get(f"{cid}_in")
    want = get(f"{cid}_out")
    what = f"case {cid} {c}"
    if op == "qsort":
        y = x.copy()
        assert fns.qsort(dtid, y.ctypes.data, n, hasnan, desc) == 0
        assert_same_sorted(y, want, what)
    elif op == "argsort":
        arg = np.zeros(n, np.uint64)
        assert fns.argsort(dtid, x.ctypes.data, arg.ctypes.data, n, hasnan, desc) == 0
        assert_arg_sorted(x, arg, x[want.astype(np.int64)], what)
    elif op == "qselect":
        y = x.copy()
        assert fns.qselect(dtid, y.ctypes.data, c["k"], n, hasnan, desc) == 0
        if n > 1:
            assert_partitioned(y, c["k"], want[c["k"]], bool(desc), what)
    elif op == "partial_qsort":
        y = x.copy()
        assert fns.partial_qsort(dtid, y.ctypes.data, c["k"], n, hasnan, desc) == 0
        if n > 1:
            assert_same_sorted(y[:c["k"]], want[:c["k"]], what)
    elif op == "argselect":
        arg = np.zeros(n, np.uint64)
        assert fns.argselect(dtid, x.ctypes.data, arg.ctypes.data, c["k"], n, hasnan) == 0
        if n > 1:
            assert_partitioned(x[arg.astype(np.int64)], c["k"], x[int(want[c["k"]])], False, what)
    else:
        v = get(f"{cid}_vin")
        wk, wv = get(f"{cid}_out"), get(f"{cid}_vout")
        y, w = x.copy(), v.copy()
        vt = DT[c["vdtype"]]
        if op == "keyvalue_qsort":
            assert fns.keyvalue_qsort(dtid, vt, y.ctypes.data, w.ctypes.data, n, hasnan, desc) == 0
            assert_same_sorted(y, wk, what)
        else:
            assert getattr(fns, op)(dtid, vt, y.ctypes.data, w.ctypes.data, c["k"], n, hasnan,
                                    desc) == 0
            if op == "keyvalue_partial_sort":
                assert_same_sorted(y[:c["k"]], wk[:c["k"]], what)
            else:
                assert_partitioned(y, c["k"], wk[c["k"]], bool(desc), what)
        assert_pairs_preserved(x, v, y, w, what)
        assert_pairs_preserved(x, v, wk, wv, what + " (golden)")

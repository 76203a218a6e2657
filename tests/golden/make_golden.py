"""Generate golden fixtures by running the reference library itself.

Run on an x86-64 host where oracle/Makefile can build the reference from its
sources (``make -C oracle ref``).  Writes tests/golden/golden.npz: for every
case the seeded input and the reference's output, packed into one byte blob
with a JSON table (see ``load`` in tests/golden_io.py).  The inputs come from
tests/xss_arrays.py (seeded restatements of utils/rand_array.h shapes).

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from oracle import pyoracle  # noqa: E402
from xss_arrays import SHAPES, KEY_TYPES, KV_TYPES, get_array, is_nan_test, kv_values  # noqa: E402

DT = {"uint16": 0, "int16": 1, "float16": 2, "uint32": 3, "int32": 4, "float32": 5,
      "uint64": 6, "int64": 7, "float64": 8}
SIZES_FULL = [1, 2, 17, 129, 300]
SIZES_BIG = [5000]
FEW_SHAPES = ["random", "smallrange", "rand_with_nan", "constant"]


def cases():
    cid = 0
    for dt in KEY_TYPES:
        for shape in SHAPES:
            for n in SIZES_FULL:
                for desc in (False, True):
                    yield cid, dict(op="qsort", dtype=dt, shape=shape, n=n, desc=desc)
                    cid += 1
                    yield cid, dict(op="argsort", dtype=dt, shape=shape, n=n, desc=desc)
                    cid += 1
            if shape in FEW_SHAPES[:3]:
                # crosses the one-CTA size limit of the GPU path
                for n in SIZES_BIG:
                    yield cid, dict(op="qsort", dtype=dt, shape=shape, n=n, desc=shape == "rand_with_nan")
                    cid += 1
            for n in SIZES_FULL:
                if shape not in FEW_SHAPES:
                    continue
                k = (n * 2) // 3
                for desc in (False, True):
                    yield cid, dict(op="qselect", dtype=dt, shape=shape, n=n, k=k, desc=desc)
                    cid += 1
                    yield cid, dict(op="partial_qsort", dtype=dt, shape=shape, n=n,
                                    k=max(1, k), desc=desc)
                    cid += 1
                yield cid, dict(op="argselect", dtype=dt, shape=shape, n=n, k=k, desc=False)
                cid += 1
    for kt in KV_TYPES:
        for vt in KV_TYPES:
            for shape in FEW_SHAPES[:3]:
                for n in [33, 150]:
                    for desc in (False, True):
                        yield cid, dict(op="keyvalue_qsort", dtype=kt, vdtype=vt, shape=shape,
                                        n=n, desc=desc)
                        cid += 1
                    yield cid, dict(op="keyvalue_select", dtype=kt, vdtype=vt, shape=shape,
                                    n=n, k=n // 3, desc=True)
                    cid += 1
                    yield cid, dict(op="keyvalue_partial_sort", dtype=kt, vdtype=vt,
                                    shape=shape, n=n, k=max(1, n // 3), desc=False)
                    cid += 1


def main():
    ref = pyoracle.reference()
    if ref is None:
        # the reference's source tree: $XSS_REFERENCE_SRC, else where this
        # fixture generator was run against it
        pyoracle.build_reference(os.environ.get("XSS_REFERENCE_SRC", "/root/reference"))
        ref = pyoracle.reference()
    if ref is None:
        sys.exit("reference library not buildable on this host")
    arrays = {}
    index = {}
    for cid, c in cases():
        dt = np.dtype(c["dtype"])
        hasnan = is_nan_test(c["shape"])
        x = get_array(c["shape"], dt, c["n"], seed=1000 + cid)
        arrays[f"{cid}_in"] = x.copy()
        op, n, desc = c["op"], c["n"], int(c["desc"])
        y = x.copy()
        if op == "qsort":
            rc = ref.qsort(DT[c["dtype"]], y.ctypes.data, n, hasnan, desc)
            arrays[f"{cid}_out"] = y
        elif op == "argsort":
            arg = np.zeros(n, np.uint64)
            rc = ref.argsort(DT[c["dtype"]], y.ctypes.data, arg.ctypes.data, n, hasnan, desc)
            arrays[f"{cid}_out"] = arg.astype(np.uint16)  # every case has n < 65536
        elif op == "qselect":
            rc = ref.qselect(DT[c["dtype"]], y.ctypes.data, c["k"], n, hasnan, desc)
            arrays[f"{cid}_out"] = y
        elif op == "partial_qsort":
            rc = ref.partial_qsort(DT[c["dtype"]], y.ctypes.data, c["k"], n, hasnan, desc)
            arrays[f"{cid}_out"] = y
        elif op == "argselect":
            arg = np.zeros(n, np.uint64)
            rc = ref.argselect(DT[c["dtype"]], y.ctypes.data, arg.ctypes.data, c["k"], n, hasnan)
            arrays[f"{cid}_out"] = arg.astype(np.uint16)
        else:
            v = kv_values(c["vdtype"], n, seed=cid)
            arrays[f"{cid}_vin"] = v.copy()
            fn = getattr(ref, op)
            if op == "keyvalue_qsort":
                rc = fn(DT[c["dtype"]], DT[c["vdtype"]], y.ctypes.data, v.ctypes.data, n,
                        hasnan, desc)
            else:
                rc = fn(DT[c["dtype"]], DT[c["vdtype"]], y.ctypes.data, v.ctypes.data, c["k"],
                        n, hasnan, desc)
            arrays[f"{cid}_out"] = y
            arrays[f"{cid}_vout"] = v
        assert rc == 0, (cid, c, rc)
        c["hasnan"] = hasnan
        index[str(cid)] = c
    # one byte blob + a JSON table of (offset, length, dtype): far smaller than
    # thousands of separate .npy members
    table, parts, off = {}, [], 0
    for name, a in arrays.items():
        b = np.ascontiguousarray(a).view(np.uint8).ravel()
        table[name] = [off, int(b.size), a.dtype.name]
        parts.append(b)
        off += b.size
    meta = json.dumps({"cases": index, "arrays": table}).encode()
    out = os.path.join(HERE, "golden.npz")
    np.savez_compressed(out, blob=np.concatenate(parts) if parts else np.zeros(0, np.uint8),
                        meta=np.frombuffer(meta, dtype=np.uint8))
    print(f"{len(index)} cases -> {out} ({os.path.getsize(out) / 1e6:.2f} MB)")


if __name__ == "__main__":
    main()

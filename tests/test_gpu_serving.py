"""Serving loop: every result in a concurrent mix equals the same request run
alone, small same-kind requests are coalesced into batched launches, a full
queue sheds requests, and shutdown drains or refuses what is queued."""
import numpy as np
import pytest

from xss_arrays import (assert_arg_sorted, assert_is_permutation, assert_pairs_preserved,
                        assert_partitioned, assert_same_sorted, get_array, kv_values, ref_sorted)

pytestmark = pytest.mark.gpu


def _pinned(torch, a):
    t = torch.empty(a.nbytes, dtype=torch.uint8, pin_memory=True)
    v = t.numpy().view(a.dtype)
    v[:] = a
    return t, v


def _mix(rng):
    ops = ["qsort", "qselect", "partial_qsort", "argsort", "argselect", "keyvalue_qsort",
           "keyvalue_select", "keyvalue_partial_sort"]
    out = []
    for i in range(160):
        op = ops[i % len(ops)]
        kv = op.startswith("keyvalue")
        dt = rng.choice(["float32", "int64", "float64", "uint32"] if kv else
                        ["float32", "int64", "float16", "float64", "uint32", "int16"])
        n = int(2 ** rng.uniform(0, 19)) if i % 5 else int(rng.integers(1, 3000))
        out.append((op, str(dt), max(n, 1), bool(rng.integers(0, 2))))
    return out


def test_results_same_alone_and_in_the_mix(xss, cuda):
    torch = cuda
    rng = np.random.default_rng(21)
    srv = xss.Server(hbm_budget_bytes=1 << 30, small_max=8192)
    keep, reqs = [], []
    for i, (op, dt, n, desc) in enumerate(_mix(rng)):
        x = get_array("mixed_special" if np.dtype(dt).kind == "f" else "random", dt, n, seed=i)
        tin, xin = _pinned(torch, x)
        tout, xout = _pinned(torch, np.zeros_like(x))
        rec = dict(op=op, dt=dt, n=n, desc=desc, x=x, xout=xout, bufs=[tin, tout])
        k = int(rng.integers(0, n)) if n > 1 else 0
        if op in ("partial_qsort", "keyvalue_partial_sort"):
            k = max(1, k)
        rec["k"] = k
        kw = dict(n=n, k=k, hasnan=True, descending=desc and op != "argselect")
        if op.startswith("keyvalue"):
            v = kv_values("uint64", n, seed=i)
            tv, vin = _pinned(torch, v)
            tvo, vout = _pinned(torch, np.zeros_like(v))
            rec.update(v=v, vout=vout)
            rec["bufs"] += [tv, tvo]
            t = srv.submit(op, dt, xin.ctypes.data, xout.ctypes.data, vals_in=vin.ctypes.data,
                           vals_out=vout.ctypes.data, val_dtype="uint64", **kw)
        elif op.startswith("arg"):
            a = torch.empty(n * 8, dtype=torch.uint8, pin_memory=True)
            rec["arg"] = a.numpy().view(np.uint64)
            rec["bufs"].append(a)
            t = srv.submit(op, dt, xin.ctypes.data, None, arg_out=rec["arg"].ctypes.data, **kw)
        else:
            t = srv.submit(op, dt, xin.ctypes.data, xout.ctypes.data, **kw)
        assert t is not None
        rec["ticket"] = t
        reqs.append(rec)
    for rec in reqs:
        assert srv.wait(rec["ticket"]) == 0, rec["op"]
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) and st["failed"] == 0
    assert st["batches"] >= 1 and st["batched_requests"] >= 2
    assert st["p99_us"] >= st["p50_us"] > 0
    for rec in reqs:
        op, x, n, desc, k = rec["op"], rec["x"], rec["n"], rec["desc"], rec["k"]
        what = f"{op} {rec['dt']} n={n} desc={desc} k={k}"
        if op == "qsort":
            alone = x.copy()
            xss.qsort(alone, True, desc)
            assert_same_sorted(rec["xout"], alone, what)
        elif op == "argsort":
            assert_arg_sorted(x, rec["arg"], ref_sorted(x, desc), what)
        elif op == "argselect":
            assert_is_permutation(rec["arg"], n, what)
            if n > 1:
                assert_partitioned(x[rec["arg"].astype(np.int64)], k, ref_sorted(x)[k], False, what)
        elif op in ("qselect", "partial_qsort"):
            if n > 1:
                want = ref_sorted(x, desc)
                if op == "qselect":
                    assert_partitioned(rec["xout"], k, want[k], desc, what)
                else:
                    assert_same_sorted(rec["xout"][:k], want[:k], what)
                assert_same_sorted(ref_sorted(rec["xout"]), ref_sorted(x), what)
        else:
            assert_pairs_preserved(x, rec["v"], rec["xout"], rec["vout"], what)
            if n > 1:
                want = ref_sorted(x, desc)
                if op == "keyvalue_qsort":
                    assert_same_sorted(rec["xout"], want, what)
                elif op == "keyvalue_select":
                    assert_partitioned(rec["xout"], k, want[k], desc, what)
                else:
                    assert_same_sorted(rec["xout"][:k], want[:k], what)


def test_full_queue_sheds_and_shutdown_drains(xss, cuda):
    torch = cuda
    # room for one 1M-key request (data + scratch) at a time: the rest queue
    srv = xss.Server(hbm_budget_bytes=12 << 20, max_queue=4, small_max=1)
    x = get_array("random", "float32", 1 << 20, seed=1)
    tin, xin = _pinned(torch, x)
    outs = [_pinned(torch, np.zeros_like(x)) for _ in range(64)]
    tickets, shed = [], 0
    for t_out, xo in outs:   # submitted back to back, far faster than they are served
        t = srv.submit("qsort", "float32", xin.ctypes.data, xo.ctypes.data, n=x.size)
        if t is None:
            shed += 1
        else:
            tickets.append((t, xo))
    assert shed > 0
    srv.close(drain=True)  # finishes everything admitted before returning
    want = np.sort(x)
    for _, xo in tickets:
        assert np.array_equal(xo, want)


def test_large_requests_use_shared_sm_lines(xss, cuda):
    """Above 2^24 keys a sort normally takes the large-array pass lines; the
    server's thread takes the mid-size lines for every size, with workspace
    sized for either.  Large requests through the server must match the same
    sorts done directly."""
    torch = cuda
    n = (1 << 24) + 4097
    rng = np.random.default_rng(31)
    srv = xss.Server(hbm_budget_bytes=4 << 30, small_max=8192)
    x = rng.standard_normal(n).astype(np.float32)
    k64 = rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, n, dtype=np.int64)
    v64 = np.arange(n, dtype=np.uint64)
    bufs = []
    tin, xin = _pinned(torch, x)
    tout, xout = _pinned(torch, np.zeros_like(x))
    tk, kin = _pinned(torch, k64)
    tko, kout = _pinned(torch, np.zeros_like(k64))
    tv, vin = _pinned(torch, v64)
    tvo, vout = _pinned(torch, np.zeros_like(v64))
    bufs += [tin, tout, tk, tko, tv, tvo]
    t1 = srv.submit("qsort", "float32", xin.ctypes.data, xout.ctypes.data, n=n)
    t2 = srv.submit("keyvalue_qsort", "int64", kin.ctypes.data, kout.ctypes.data,
                    vals_in=vin.ctypes.data, vals_out=vout.ctypes.data, val_dtype="uint64", n=n)
    assert t1 is not None and t2 is not None
    assert srv.wait(t1) == 0 and srv.wait(t2) == 0
    srv.close()
    assert np.array_equal(xout, np.sort(x))
    assert np.array_equal(kout, np.sort(k64))
    assert np.array_equal(k64[vout.astype(np.int64)], kout)

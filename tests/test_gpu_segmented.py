"""Batched segmented sort against the oracle, segment by segment.

Every size class is exercised (empty and one-key segments, warp-sized,
CTA-sized, and segments large enough for the segmented radix sort), through
the one-shot entry point, a reusable plan, and a plan replayed as a CUDA graph.
"""
import numpy as np
import pytest

from golden_io import DT
from xss_arrays import (assert_pairs_preserved, assert_same_sorted, get_array, kv_values,
                        ref_sorted)

pytestmark = pytest.mark.gpu

FIXED = [0, 1, 2, 3, 17, 31, 32, 33, 100, 255, 256, 257, 1000, 4095, 4096, 4097, 5000, 20000,
         70001]


def _layout(seed, count=300, hi=17):
    rng = np.random.default_rng(seed)
    sizes = np.concatenate([np.array(FIXED), np.floor(2.0 ** rng.uniform(0, hi, count))])
    rng.shuffle(sizes)
    off = np.zeros(sizes.size + 1, np.uint64)
    off[1:] = np.cumsum(sizes.astype(np.uint64))
    return off


def _make(kdt, vdt, off, seed):
    n = int(off[-1])
    shape = "mixed_special" if np.dtype(kdt).kind == "f" else "random"
    k = get_array(shape, kdt, n, seed)
    v = kv_values(vdt, n, seed) if vdt else None
    return k, v


def _check(k_in, v_in, k_out, v_out, off, desc, what):
    for i in range(off.size - 1):
        b, e = int(off[i]), int(off[i + 1])
        if e - b == 0:
            continue
        assert_same_sorted(k_out[b:e], ref_sorted(k_in[b:e], desc), f"{what} seg {i} [{b},{e})")
        if v_in is not None:
            assert_pairs_preserved(k_in[b:e], v_in[b:e], k_out[b:e], v_out[b:e], f"{what} seg {i}")


def _dev(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a).view(np.uint8).copy()).cuda()


@pytest.mark.parametrize("kdt,vdt", [("int32", "uint32"), ("float32", "uint32"),
                                     ("float64", None), ("uint16", None), ("int64", "uint64"),
                                     ("float32", None), ("uint64", "float32"),
                                     ("float32", "uint16"), ("uint16", "float16"),
                                     ("int64", "int16")])
@pytest.mark.parametrize("desc", [False, True])
def test_segmented_matches_oracle(xss, cuda, kdt, vdt, desc):
    torch = cuda
    off = _layout(hash((kdt, vdt, desc)) % 1000)
    k, v = _make(kdt, vdt, off, 5)
    hasnan = np.dtype(kdt).kind == "f"
    dk, dv = _dev(torch, k), (_dev(torch, v) if vdt else None)
    doff = torch.from_numpy(off.view(np.int64).copy()).cuda()
    wsb = xss.segmented_workspace_size(kdt, vdt, off)
    ws = torch.empty(max(wsb, 1), dtype=torch.uint8, device="cuda")
    xss.gpu_segmented_sort(kdt, vdt, dk.data_ptr(), dv.data_ptr() if vdt else 0, doff.data_ptr(),
                           off, off.size - 1, hasnan, desc, ws.data_ptr(), wsb)
    xss.stream_status()
    ko = dk.cpu().numpy().view(k.dtype)
    vo = dv.cpu().numpy().view(v.dtype) if vdt else None
    _check(k, v, ko, vo, off, desc, f"one-shot {kdt}/{vdt}")


def test_plan_and_graph_replay(xss, cuda):
    torch = cuda
    off = _layout(7, count=500)
    plan = xss.SegPlan("int32", "uint32", off)
    wsb = plan.workspace_size
    ws = torch.empty(wsb, dtype=torch.uint8, device="cuda")
    doff = torch.from_numpy(off.view(np.int64).copy()).cuda()
    n = int(off[-1])
    dk = torch.empty(n * 4, dtype=torch.uint8, device="cuda")
    dv = torch.empty(n * 4, dtype=torch.uint8, device="cuda")
    for rep, use_graph in enumerate([False, True, True, True]):
        k, v = _make("int32", "uint32", off, 100 + rep)
        dk.copy_(torch.from_numpy(k.view(np.uint8)))
        dv.copy_(torch.from_numpy(v.view(np.uint8)))
        plan.run(dk.data_ptr(), dv.data_ptr(), doff.data_ptr(), ws.data_ptr(), wsb,
                 use_graph=use_graph)
        xss.stream_status()
        _check(k, v, dk.cpu().numpy().view(np.int32), dv.cpu().numpy().view(np.uint32), off,
               False, f"plan rep {rep} graph={use_graph}")
    plan.close()


def test_percall_baseline_agrees(xss, cuda):
    torch = cuda
    off = _layout(9, count=60, hi=15)
    k, v = _make("int32", "uint32", off, 3)
    dk, dv = _dev(torch, k), _dev(torch, v)
    xss.gpu_segmented_sort_percall("int32", "uint32", dk.data_ptr(), dv.data_ptr(), off)
    xss.stream_status()
    _check(k, v, dk.cpu().numpy().view(np.int32), dv.cpu().numpy().view(np.uint32), off, False,
           "per-call")


@pytest.mark.parametrize("shape", ["constant", "smallrange", "sorted", "reverse", "random_5d"])
@pytest.mark.parametrize("kdt,vdt", [("int32", "uint32"), ("uint64", None), ("float16", "uint64")])
def test_segmented_mid_sizes_shapes(xss, cuda, shape, kdt, vdt):
    """Segments of 257..4096 keys (one CTA each, radix sort in shared memory)
    with inputs whose digits repeat: passes whose digit every key shares are
    skipped, the others must keep the order stable."""
    torch = cuda
    rng = np.random.default_rng(31)
    sizes = np.concatenate([[257, 300, 511, 512, 513, 1024, 1025, 2047, 4095, 4096],
                            rng.integers(257, 4097, 40)]).astype(np.uint64)
    off = np.zeros(sizes.size + 1, np.uint64)
    off[1:] = np.cumsum(sizes)
    n = int(off[-1])
    k = np.concatenate([get_array(shape, kdt, int(s), 7 + i) for i, s in enumerate(sizes)])
    v = kv_values(vdt, n, 4) if vdt else None
    hasnan = np.dtype(kdt).kind == "f"
    for desc in (False, True):
        dk, dv = _dev(torch, k), (_dev(torch, v) if vdt else None)
        doff = torch.from_numpy(off.view(np.int64).copy()).cuda()
        xss.gpu_segmented_sort(kdt, vdt, dk.data_ptr(), dv.data_ptr() if vdt else 0,
                               doff.data_ptr(), off, off.size - 1, hasnan, desc)
        xss.stream_status()
        ko = dk.cpu().numpy().view(k.dtype)
        vo = dv.cpu().numpy().view(v.dtype) if vdt else None
        _check(k, v, ko, vo, off, desc, f"{shape} {kdt}/{vdt} desc={desc}")
        if vdt:
            # stable: values of equal keys keep their input order
            for i in range(sizes.size):
                b, e = int(off[i]), int(off[i + 1])
                kk = k[b:e]
                order = np.argsort(-kk.astype(np.float64) if desc else kk, kind="stable")
                if np.dtype(kdt).kind != "f":
                    assert np.array_equal(vo[b:e], v[b:e][order]), f"{shape} seg {i} stability"


@pytest.mark.parametrize("kdt,vdt", [("float32", "uint32"), ("int64", None), ("uint16", "uint16")])
@pytest.mark.parametrize("k", [1, 7, 300, 5000])
def test_segmented_topk(xss, cuda, kdt, vdt, k):
    """Each segment's first min(k, len) positions: its k smallest (largest when
    descending) in order, pairs kept; the segment as a whole a permutation."""
    torch = cuda
    for desc in (False, True):
        off = _layout(k + 31 * desc)
        keys, vals = _make(kdt, vdt, off, 9)
        hasnan = np.dtype(kdt).kind == "f"
        dk, dv = _dev(torch, keys), (_dev(torch, vals) if vdt else None)
        doff = _dev(torch, off)
        xss.gpu_segmented_topk(kdt, vdt, dk.data_ptr(), dv.data_ptr() if vdt else 0,
                               doff.data_ptr(), off, off.size - 1, k, hasnan, desc)
        xss.stream_status()
        ko = dk.cpu().numpy().view(keys.dtype)
        vo = dv.cpu().numpy().view(vals.dtype) if vdt else None
        for i in range(off.size - 1):
            b, e = int(off[i]), int(off[i + 1])
            if e == b:
                continue
            m = min(k, e - b)
            what = f"topk {kdt}/{vdt} k={k} desc={desc} seg {i}"
            assert_same_sorted(ko[b:b + m], ref_sorted(keys[b:e], desc)[:m], what)
            assert_same_sorted(ref_sorted(ko[b:e]), ref_sorted(keys[b:e]), what + " multiset")
            if vdt:
                assert_pairs_preserved(keys[b:e], vals[b:e], ko[b:e], vo[b:e], what)


@pytest.mark.parametrize("shape", ["reverse", "sorted", "constant", "smallrange"])
@pytest.mark.parametrize("k", [1, 1000, 2048, 2049])
def test_segmented_topk_streamed_shapes(xss, cuda, shape, k):
    """Segments above 4096 keys take the streamed top-k for k <= 2048 (one read
    of the segment, keys below the running k-th staged and merged on chip) and
    the full segmented sort above it.  Reversed input (sorted input when
    descending) makes every key a candidate and merges every window; constant
    input stages nothing."""
    torch = cuda
    sizes = [0, 1, 100, 4096, 4097, 6000, 6144, 10000, 65536, 130001, 5000, 8193]
    off = np.zeros(len(sizes) + 1, np.uint64)
    off[1:] = np.cumsum(np.array(sizes, dtype=np.uint64))
    n = int(off[-1])
    for kdt, vdt in (("int32", "uint32"), ("float64", None), ("uint16", "uint64")):
        keys = get_array(shape, kdt, n, 17)
        vals = kv_values(vdt, n, 17) if vdt else None
        for desc in (False, True):
            dk, dv = _dev(torch, keys), (_dev(torch, vals) if vdt else None)
            doff = _dev(torch, off)
            xss.gpu_segmented_topk(kdt, vdt, dk.data_ptr(), dv.data_ptr() if vdt else 0,
                                   doff.data_ptr(), off, off.size - 1, k, False, desc)
            xss.stream_status()
            ko = dk.cpu().numpy().view(keys.dtype)
            vo = dv.cpu().numpy().view(vals.dtype) if vdt else None
            for i in range(off.size - 1):
                b, e = int(off[i]), int(off[i + 1])
                if e == b:
                    continue
                m = min(k, e - b)
                what = f"topk {shape} {kdt}/{vdt} k={k} desc={desc} seg {i} len {e - b}"
                assert_same_sorted(ko[b:b + m], ref_sorted(keys[b:e], desc)[:m], what)
                assert_same_sorted(ref_sorted(ko[b:e]), ref_sorted(keys[b:e]), what + " multiset")
                if vdt:
                    assert_pairs_preserved(keys[b:e], vals[b:e], ko[b:e], vo[b:e], what)

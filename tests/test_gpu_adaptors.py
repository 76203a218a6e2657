"""Framework adaptors (torch.sort-style on CUDA tensors, NumPy-style on host
arrays) against torch and NumPy themselves, and the device record sort
against a stable host sort."""
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "x86-simd-sort_gb300"))


@pytest.fixture(scope="module")
def ad(xss):
    import adaptors
    return adaptors


def _same(torch, a, b):
    return bool(((a == b) | (torch.isnan(a) & torch.isnan(b))).all()) if a.is_floating_point() \
        else bool((a == b).all())


@pytest.mark.parametrize("dtype", ["float32", "float64", "float16", "int32", "int64", "int16"])
@pytest.mark.parametrize("descending", [False, True])
def test_torch_sort_1d_matches_stable_torch_sort(ad, cuda, dtype, descending):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(5)
    n = 300_001
    if dtype.startswith("float"):
        x = torch.randn(n, device="cuda", generator=g).to(getattr(torch, dtype))
        x[torch.rand(n, device="cuda", generator=g) < 0.01] = float("nan")
        x[x == 0] = 1.0   # keep -0.0 / +0.0 out: the frameworks call them equal
    else:
        x = torch.randint(-50, 50, (n,), device="cuda", generator=g).to(getattr(torch, dtype))
    v, i = ad.sort(x, descending=descending)
    rv, ri = torch.sort(x, descending=descending, stable=True)
    torch.cuda.synchronize()
    assert _same(torch, v, rv)
    assert torch.equal(i, ri)


@pytest.mark.parametrize("dtype", ["float32", "int64", "float16"])
def test_torch_sort_rows_matches_torch(ad, cuda, dtype):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(6)
    x = torch.randint(-1000, 1000, (257, 3001), device="cuda", generator=g).to(getattr(torch, dtype))
    for desc in (False, True):
        v, i = ad.sort(x, descending=desc)
        rv, ri = torch.sort(x, dim=-1, descending=desc, stable=True)
        assert torch.equal(v, rv) and torch.equal(i, ri)
    assert torch.equal(ad.argsort(x), torch.argsort(x, dim=-1, stable=True))


def test_torch_kthvalue_and_topk(ad, cuda):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(7)
    x = torch.randn(1 << 20, device="cuda", generator=g)
    for k in (1, 1000, 1 << 19):
        val, idx = ad.kthvalue(x, k)
        assert float(val) == float(torch.kthvalue(x, k).values)
        assert float(x[idx]) == float(val)
    for largest in (True, False):
        v, i = ad.topk(x, 4096, largest=largest)
        rv = torch.topk(x, 4096, largest=largest, sorted=True).values
        assert torch.equal(v, rv) and torch.equal(x[i], v)
    h = x.to(torch.float16)
    v, i = ad.topk(h, 100)
    assert torch.equal(v, torch.topk(h, 100).values) and torch.equal(h[i], v)


def test_numpy_entry_points(ad, cuda):
    rng = np.random.default_rng(8)
    a = rng.standard_normal(500_000).astype(np.float32)
    a[rng.random(a.size) < 0.001] = np.nan
    assert np.array_equal(ad.np_sort(a), np.sort(a), equal_nan=True)
    b = rng.integers(0, 1000, 400_000).astype(np.int32)
    assert np.array_equal(ad.np_argsort(b), np.argsort(b, kind="stable"))
    for kth in (0, 12345, b.size - 1):
        p = ad.np_partition(b, kth)
        assert p[kth] == np.partition(b, kth)[kth]
        assert (p[:kth] <= p[kth]).all() and (p[kth + 1:] >= p[kth]).all()
        ap = ad.np_argpartition(b, kth)
        assert b[ap[kth]] == p[kth] and np.array_equal(np.sort(ap), np.arange(b.size))
    assert ad.np_sort(np.array([], dtype=np.float64)).size == 0
    assert ad.np_argsort(np.array([3.0])).tolist() == [0]


REC = np.dtype([("x", "<i4"), ("y", "<i4"), ("distance", "<f4"), ("metric", "<u8")], align=True)


@pytest.mark.parametrize("field,kdt,desc", [("metric", "uint64", False), ("distance", "float32", True),
                                            ("x", "int32", False)])
def test_device_record_sort(xss, cuda, field, kdt, desc):
    torch = cuda
    rng = np.random.default_rng(9)
    n = 250_000
    recs = np.zeros(n, dtype=REC)
    recs["x"] = rng.integers(-100, 100, n)
    recs["y"] = np.arange(n)
    recs["distance"] = rng.standard_normal(n).astype(np.float32)
    recs["metric"] = rng.integers(0, 3000, n)
    raw = recs.view(np.uint8)
    d = torch.from_numpy(raw.copy()).cuda()
    xss.gpu_object_qsort(d.data_ptr(), n, REC.itemsize, REC.fields[field][1], kdt, False, desc,
                         stream=torch.cuda.current_stream().cuda_stream)
    xss.stream_status(torch.cuda.current_stream().cuda_stream)
    got = d.cpu().numpy().view(REC)
    key = recs[field]
    order = np.argsort(-key if desc else key, kind="stable")
    assert np.array_equal(got, recs[order])


def test_device_record_sort_rejects_bad_layout(xss, cuda):
    torch = cuda
    d = torch.zeros(64, dtype=torch.uint8, device="cuda")
    with pytest.raises(xss.XssError):
        xss.gpu_object_qsort(d.data_ptr(), 4, 16, 12, "uint64")       # key past the record
    with pytest.raises(xss.XssError):
        xss.gpu_object_qsort(d.data_ptr(), 4, 16, 0, "uint16")        # 16-bit keys: unsupported


@pytest.mark.parametrize("kdt", ["uint16", "int16", "float16"])
@pytest.mark.parametrize("vdt", ["uint32", "uint64"])
def test_keyvalue_16bit_keys(xss, cuda, kdt, vdt):
    """16-bit keys carrying 32/64-bit values (not offered by the reference):
    keys in the order of a stable sort, values still attached to their keys."""
    torch = cuda
    rng = np.random.default_rng(10)
    n = 1_000_003
    if kdt == "float16":
        k0 = rng.standard_normal(n).astype(np.float16)
        k0[rng.random(n) < 0.001] = np.nan
        k0[k0 == 0] = 1.0
    else:
        k0 = rng.integers(np.iinfo(kdt).min, np.iinfo(kdt).max, n, endpoint=True).astype(kdt)
    tv = {"uint32": torch.int32, "uint64": torch.int64}[vdt]
    for desc in (False, True):
        keys = torch.from_numpy(k0.view(np.int16).copy()).cuda()
        vals = torch.arange(n, dtype=tv, device="cuda")
        xss.gpu_keyvalue_qsort(kdt, vdt, keys.data_ptr(), vals.data_ptr(), n, True, desc)
        xss.stream_status()
        got_v = vals.cpu().numpy().astype(np.int64)
        order = np.argsort(-k0.astype(np.float64) if desc else k0, kind="stable")
        if kdt == "float16":   # NaN last ascending, first descending
            nan = np.isnan(k0)
            fin = np.flatnonzero(~nan)
            fo = fin[np.argsort(-k0[fin].astype(np.float64) if desc else k0[fin], kind="stable")]
            order = np.concatenate([np.flatnonzero(nan), fo] if desc else [fo, np.flatnonzero(nan)])
        assert np.array_equal(got_v, order)
        assert np.array_equal(keys.cpu().numpy().view(kdt).view(np.uint16),
                              k0[order].view(np.uint16))
    # select: the k-th key in place, values still attached
    keys = torch.from_numpy(k0.view(np.int16).copy()).cuda()
    vals = torch.arange(n, dtype=tv, device="cuda")
    kk = 4321
    xss.gpu_keyvalue_select(kdt, vdt, keys.data_ptr(), vals.data_ptr(), kk, n, True)
    xss.stream_status()
    kv = keys.cpu().numpy().view(kdt)
    assert np.array_equal(kv.view(np.uint16), k0[vals.cpu().numpy().astype(np.int64)].view(np.uint16))
    assert kv[kk] == np.sort(k0)[kk] or (np.isnan(kv[kk]) and np.isnan(np.sort(k0)[kk]))

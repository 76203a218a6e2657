"""Full-size checks at the benchmark configurations, through size-independent
properties checked on the device (the oracle is too slow at these sizes):
sortedness, permutation validity, gathered keys, the partition property, and
equality with torch.sort where torch's order is the same as the reference's
(no NaN)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N28 = 1 << 28
N27 = 1 << 27


def _perm_ok(torch, idx, n):
    seen = torch.zeros(n, dtype=torch.int32, device="cuda")
    seen.index_add_(0, idx, torch.ones(n, dtype=torch.int32, device="cuda"))
    return bool((seen == 1).all())


def test_qsort_f32_2e28(xss, cuda):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.rand(N28, device="cuda", generator=g) * 2 - 1
    y = x.clone()
    xss.gpu_qsort("float32", y.data_ptr(), N28)
    xss.stream_status()
    assert torch.equal(y, torch.sort(x).values)


def test_keyvalue_int64_uint64_2e28(xss, cuda):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(1)
    k0 = torch.randint(0, 256, (N28 * 8,), dtype=torch.uint8, device="cuda",
                       generator=g).view(torch.int64)
    k, v = k0.clone(), torch.arange(N28, dtype=torch.int64, device="cuda")
    xss.gpu_keyvalue_qsort("int64", "uint64", k.data_ptr(), v.data_ptr(), N28)
    xss.stream_status()
    assert bool((k[1:] >= k[:-1]).all())
    assert bool((k0[v] == k).all())
    assert _perm_ok(torch, v, N28)


def test_argsort_int64_2e28(xss, cuda):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(1)
    k = torch.randint(0, 256, (N28 * 8,), dtype=torch.uint8, device="cuda",
                      generator=g).view(torch.int64)
    arg = torch.empty(N28, dtype=torch.int64, device="cuda")
    xss.gpu_argsort("int64", k.data_ptr(), arg.data_ptr(), N28)
    xss.stream_status()
    assert _perm_ok(torch, arg, N28)
    s = k[arg]
    assert bool((s[1:] >= s[:-1]).all())


def test_argsort_f64_nan_zeros_desc_2e28(xss, cuda):
    """1% quiet NaN, 0.25% +0.0 and 0.25% -0.0, hasnan, descending."""
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(1)
    x = torch.randn(N28, dtype=torch.float64, device="cuda", generator=g)
    u = torch.rand(N28, dtype=torch.float64, device="cuda", generator=g)
    x[u < 0.01] = float("nan")
    x[(u >= 0.01) & (u < 0.0125)] = 0.0
    x[(u >= 0.0125) & (u < 0.015)] = -0.0
    arg = torch.empty(N28, dtype=torch.int64, device="cuda")
    xss.gpu_argsort("float64", x.data_ptr(), arg.data_ptr(), N28, True, True)
    xss.stream_status()
    assert _perm_ok(torch, arg, N28)
    s = x[arg]
    nan = torch.isnan(s)
    cnt = int(nan.sum())
    assert cnt == int(torch.isnan(x).sum()) and bool(nan[:cnt].all())
    rest = s[cnt:]
    assert bool((rest[1:] <= rest[:-1]).all())   # -0.0 == +0.0 compare equal


@pytest.mark.parametrize("k", [1, 1000, 1 << 26])
def test_qselect_partial_f32_2e27(xss, cuda, k):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(2)
    x = torch.randn(N27, device="cuda", generator=g)
    kth = torch.kthvalue(x, k + 1).values
    y = x.clone()
    xss.gpu_qselect("float32", y.data_ptr(), k, N27)
    xss.stream_status()
    assert float(y[k]) == float(kth)
    if k:
        assert bool((y[:k] <= y[k]).all())
    assert bool((y[k + 1:] >= y[k]).all())
    z = x.clone()
    xss.gpu_partial_qsort("float32", z.data_ptr(), k, N27)
    xss.stream_status()
    assert torch.equal(z[:k], torch.sort(x).values[:k])


@pytest.mark.parametrize("dtype", ["uint16", "float16"])
def test_select_zipf_16bit_2e28(xss, cuda, dtype):
    """Zipf(s=1.1) over 4096 distinct values (heavy duplicates), k = 2^20."""
    torch = cuda
    rng = np.random.default_rng(2)
    if dtype == "uint16":
        vals = rng.choice(65536, 4096, replace=False).astype(np.uint16)
    else:
        pool = np.arange(65536, dtype=np.uint16)
        finite = pool[((pool & 0x7C00) != 0x7C00) & (pool != 0x8000)]
        vals = rng.choice(finite, 4096, replace=False).astype(np.uint16)
    p = 1.0 / np.arange(1, 4097) ** 1.1
    cdf = torch.tensor(np.cumsum(p / p.sum()), device="cuda")
    g = torch.Generator(device="cuda").manual_seed(2)
    r = torch.searchsorted(cdf, torch.rand(N28, dtype=torch.float64, device="cuda", generator=g))
    r = r.clamp(max=4095)
    x = torch.tensor(vals.view(np.int16), device="cuda")[r]          # raw 16-bit patterns
    k = 1 << 20
    y = x.clone()
    xss.gpu_qselect(dtype, y.data_ptr(), k, N28)
    xss.stream_status()
    # order-preserving view of the bits to check with torch
    if dtype == "uint16":
        key = lambda t: t.to(torch.int32) & 0xFFFF  # noqa: E731
    else:
        key = lambda t: t.view(torch.float16).to(torch.float32)  # noqa: E731
    kx = key(x)
    kth = torch.kthvalue(kx, k + 1).values
    ky = key(y)
    assert float(ky[k]) == float(kth)
    assert bool((ky[:k] <= ky[k]).all()) and bool((ky[k + 1:] >= ky[k]).all())
    assert torch.equal(torch.sort(ky).values, torch.sort(kx).values)


def test_keyvalue_partial_int32_2e27(xss, cuda):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(2)
    k0 = torch.randint(-2**31, 2**31 - 1, (N27,), dtype=torch.int32, device="cuda", generator=g)
    v0 = torch.arange(N27, dtype=torch.int32, device="cuda")
    k, v = k0.clone(), v0.clone()
    kk = 4096
    xss.gpu_keyvalue_partial_sort("int32", "uint32", k.data_ptr(), v.data_ptr(), kk, N27)
    xss.stream_status()
    assert torch.equal(k[:kk], torch.sort(k0).values[:kk])
    assert bool((k[kk:] >= k[kk - 1]).all())
    assert bool((k0[v.long()] == k).all()) and _perm_ok(torch, v.long(), N27)


def test_keyvalue_select_f32_index_2e27(xss, cuda):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(2)
    k0 = torch.randn(N27, device="cuda", generator=g)
    k, v = k0.clone(), torch.arange(N27, dtype=torch.int32, device="cuda")
    kk = 1000
    xss.gpu_keyvalue_select("float32", "uint32", k.data_ptr(), v.data_ptr(), kk, N27)
    xss.stream_status()
    assert float(k[kk]) == float(torch.kthvalue(k0, kk + 1).values)
    assert bool((k[:kk] <= k[kk]).all()) and bool((k[kk + 1:] >= k[kk]).all())
    assert bool((k0[v.long()] == k).all())


@pytest.mark.parametrize("shape", ["uniform", "smallrange"])
def test_qsort_int64_2e29_histogram_flushes(xss, cuda, shape):
    """2^29 64-bit keys: each histogram thread counts more keys than its 16-bit
    counter columns hold at once, so the counters are flushed mid-run; with a
    few distinct values every key of a column lands on the same counters."""
    torch = cuda
    n = 1 << 29
    g = torch.Generator(device="cuda").manual_seed(6)
    if shape == "uniform":
        x = torch.randint(0, 256, (n * 8,), dtype=torch.uint8, device="cuda",
                          generator=g).view(torch.int64)
    else:
        x = torch.randint(-3, 4, (n,), dtype=torch.int64, device="cuda", generator=g)
    y = x.clone()
    xss.gpu_qsort("int64", y.data_ptr(), n)
    xss.stream_status()
    assert bool((y[1:] >= y[:-1]).all())
    if shape == "smallrange":
        assert torch.equal(torch.bincount(y + 3, minlength=7), torch.bincount(x + 3, minlength=7))
    else:
        assert torch.equal(y, torch.sort(x).values)

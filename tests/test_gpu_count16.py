"""16-bit keys-only sorts by counting (csrc/xss_count16.cu), edge cases the
shape sweep does not reach: arrays that start off a 16-byte boundary, one
code repeated past a CTA's 16-bit counter (the overflow move), codes far
apart (long runs of empty codes), NaN payload rules (qsort with hasnan
writes the canonical quiet NaN 0x7c01; qselect keeps every bit pattern;
partial_qsort canonicalises only the sorted prefix), against the oracle."""
import numpy as np
import pytest

from golden_io import DT

pytestmark = pytest.mark.gpu

F16_QNAN = 0x7C01


def _dev(torch, host_u16, pad):
    """Device copy of host_u16 starting `pad` elements into a fresh buffer."""
    buf = torch.zeros(host_u16.size + 8, dtype=torch.int16, device="cuda")
    buf[pad:pad + host_u16.size] = torch.from_numpy(host_u16.view(np.int16)).cuda()
    return buf, buf.data_ptr() + 2 * pad


def _back(buf, pad, n):
    return buf[pad:pad + n].cpu().numpy().view(np.uint16)


def _oracle_sorted(oracle, x_bits, dtype, hasnan, desc):
    want = x_bits.copy()
    assert oracle.qsort(DT[dtype], want.ctypes.data, want.size, int(hasnan), int(desc)) == 0
    return want


@pytest.mark.parametrize("pad", range(8))
@pytest.mark.parametrize("dtype", ["uint16", "int16", "float16"])
def test_unaligned_starts(xss, oracle, cuda, dtype, pad):
    rng = np.random.default_rng(100 + pad)
    n = 100_003
    x = rng.integers(0, 65536, n, dtype=np.uint16)
    if dtype == "float16":
        x[(x & 0x7C00) == 0x7C00] = 0x3C00       # no NaN / inf here: plain order
    for desc in (False, True):
        buf, ptr = _dev(cuda, x, pad)
        xss.gpu_qsort(dtype, ptr, n, False, desc)
        xss.stream_status()
        got = _back(buf, pad, n)
        want = _oracle_sorted(oracle, x.view(np.dtype(dtype)).copy().view(np.uint16), dtype,
                              False, desc)
        if dtype == "float16":
            # -0 and +0 compare equal in the reference: compare their class
            zero = lambda a: np.where((a & 0x7FFF) == 0, 0, a)  # noqa: E731
            assert np.array_equal(zero(got), zero(want)), (pad, desc)
        else:
            assert np.array_equal(got, want), (pad, desc)
        # the padding around the array is untouched
        assert int(buf[:pad].abs().sum()) == 0 and int(buf[pad + n:].abs().sum()) == 0


def test_counter_overflow_and_sparse_codes(xss, cuda):
    torch = cuda
    n = 1 << 22
    # one code everywhere: every CTA's counter passes 0x8000 many times
    x = torch.full((n,), 12345, dtype=torch.int32, device="cuda").to(torch.int16)
    xss.gpu_qsort("uint16", x.data_ptr(), n)
    xss.stream_status()
    assert bool((x == 12345).all())
    # two codes at opposite ends plus one in the middle: long runs of empty codes
    g = torch.Generator(device="cuda").manual_seed(7)
    r = torch.randint(0, 3, (n,), device="cuda", generator=g)
    vals = torch.tensor([0, 40000 - 65536, -1], dtype=torch.int16, device="cuda")
    x = vals[r]
    cnt = [int((r == i).sum()) for i in range(3)]
    xss.gpu_qsort("uint16", x.data_ptr(), n)
    xss.stream_status()
    u = x.to(torch.int32) & 0xFFFF
    assert bool((u[:cnt[0]] == 0).all())
    assert bool((u[cnt[0]:cnt[0] + cnt[1]] == 40000).all())
    assert bool((u[cnt[0] + cnt[1]:] == 65535).all())


def _f16_with_nans(rng, n):
    x = rng.standard_normal(n).astype(np.float16).view(np.uint16)
    nan_at = rng.random(n) < 0.01
    payload = rng.integers(1, 0x400, n, dtype=np.uint16)
    sign = (rng.random(n) < 0.5).astype(np.uint16) << 15
    x[nan_at] = (0x7C00 | payload[nan_at] | sign[nan_at])
    return x


@pytest.mark.parametrize("desc", [False, True])
def test_f16_nan_rules(xss, cuda, desc):
    torch = cuda
    rng = np.random.default_rng(11)
    n = 300_001
    x = _f16_with_nans(rng, n)
    isnan = lambda a: (a & 0x7FFF) > 0x7C00  # noqa: E731
    cnt = int(isnan(x).sum())
    finite_sorted = np.sort(x[~isnan(x)].view(np.float16).astype(np.float32))
    if desc:
        finite_sorted = finite_sorted[::-1]

    # qsort with hasnan: canonical quiet NaNs at the end (asc) or front (desc)
    buf, ptr = _dev(torch, x, 0)
    xss.gpu_qsort("float16", ptr, n, True, desc)
    xss.stream_status()
    got = _back(buf, 0, n)
    nan_part = got[:cnt] if desc else got[n - cnt:]
    rest = got[cnt:] if desc else got[:n - cnt]
    assert (nan_part == F16_QNAN).all()
    assert np.array_equal(rest.view(np.float16).astype(np.float32), finite_sorted)

    # qselect keeps every bit pattern (NaN payloads and signs included)
    k = n // 3
    buf, ptr = _dev(torch, x, 0)
    xss.gpu_qselect("float16", ptr, k, n, True, desc)
    xss.stream_status()
    got = _back(buf, 0, n)
    assert np.array_equal(np.sort(got), np.sort(x))

    # partial_qsort: NaNs of the sorted prefix canonical, the tail's as they were
    kk = n - cnt // 2 if not desc else cnt // 2
    buf, ptr = _dev(torch, x, 0)
    xss.gpu_partial_qsort("float16", ptr, kk, n, True, desc)
    xss.stream_status()
    got = _back(buf, 0, n)
    pre, tail = got[:kk], got[kk:]
    assert (pre[isnan(pre)] == F16_QNAN).all()
    tail_nans = np.sort(tail[isnan(tail)])
    assert tail_nans.size > 0
    src_nans = x[isnan(x)]
    # every tail NaN is one of the input's NaN patterns
    assert np.isin(tail_nans, src_nans).all()

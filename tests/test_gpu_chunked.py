"""Arrays above one radix sort's size (2^30 - 1 keys) are sorted in chunks
and merged.  Parity of that path against the oracle at small sizes (a child
process with the chunk length lowered to 8192 keys), and full-size checks
above 2^30 keys: sortedness and the key multiset (qsort uint32 at 2^31 +
12345), the gathered keys and the permutation (keyvalue_qsort int64 -> uint64
at 2^30 + 1, argsort int64 at 2^30 + 7)."""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def test_chunked_path_matches_oracle(xss, cuda):
    env = dict(os.environ, XSS_MERGE_CHUNK="8192")
    r = subprocess.run([sys.executable, os.path.join(HERE, "chunked_cases.py")], env=env,
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True,
                       timeout=1800)
    assert r.returncode == 0, r.stdout[-4000:]
    assert "0 failures" in r.stdout


def _perm_ok(torch, idx, n):
    seen = torch.zeros(n, dtype=torch.int32, device="cuda")
    seen.index_add_(0, idx, torch.ones(n, dtype=torch.int32, device="cuda"))
    return bool((seen == 1).all())


def test_qsort_uint32_2e31_plus(xss, cuda):
    torch = cuda
    n = (1 << 31) + 12345
    g = torch.Generator(device="cuda").manual_seed(9)
    x = torch.randint(0, 256, (n * 4,), dtype=torch.uint8, device="cuda",
                      generator=g).view(torch.int32)
    # the key multiset: histogram of the top 16 bits and sum of the low 16 bits
    top0 = torch.bincount(((x.to(torch.int64) >> 16) & 0xFFFF), minlength=1 << 16)
    low0 = int((x.to(torch.int64) & 0xFFFF).sum())
    xss.gpu_qsort("uint32", x.data_ptr(), n)
    xss.stream_status()
    u = x.to(torch.int64) & 0xFFFFFFFF        # the keys as unsigned values
    assert bool((u[1:] >= u[:-1]).all())
    assert torch.equal(torch.bincount((u >> 16) & 0xFFFF, minlength=1 << 16), top0)
    assert int((u & 0xFFFF).sum()) == low0


def test_keyvalue_int64_uint64_2e30_plus_1(xss, cuda):
    torch = cuda
    n = (1 << 30) + 1
    g = torch.Generator(device="cuda").manual_seed(10)
    k0 = torch.randint(0, 256, (n * 8,), dtype=torch.uint8, device="cuda",
                       generator=g).view(torch.int64)
    k, v = k0.clone(), torch.arange(n, dtype=torch.int64, device="cuda")
    xss.gpu_keyvalue_qsort("int64", "uint64", k.data_ptr(), v.data_ptr(), n)
    xss.stream_status()
    assert bool((k[1:] >= k[:-1]).all())
    assert bool((k0[v] == k).all())
    assert _perm_ok(torch, v, n)


def test_argsort_int64_2e30_plus_7(xss, cuda):
    torch = cuda
    n = (1 << 30) + 7
    g = torch.Generator(device="cuda").manual_seed(11)
    k = torch.randint(-1000, 1000, (n,), dtype=torch.int64, device="cuda", generator=g)
    arg = torch.empty(n, dtype=torch.int64, device="cuda")
    xss.gpu_argsort("int64", k.data_ptr(), arg.data_ptr(), n)
    xss.stream_status()
    assert _perm_ok(torch, arg, n)
    s = k[arg]
    assert bool((s[1:] >= s[:-1]).all())
    # stable: equal keys keep their original order
    same = s[1:] == s[:-1]
    assert bool((arg[1:][same] > arg[:-1][same]).all())

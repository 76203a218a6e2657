"""Framework-facing entry points over the C ABI: torch.sort-style functions on
CUDA tensors and NumPy-style functions on host arrays.

x86-simd-sort's downstream callers are NumPy (np.sort / argsort / partition /
argpartition) and PyTorch (torch.sort / argsort); these functions give those
call shapes on the GB300 library.  NaN handling follows both frameworks: NaN
orders after every number (first when descending).  Every GPU function runs on
torch's current CUDA stream; nothing falls back to a CPU sort.

Differences worth knowing: indices come from a stable sort (equal keys keep
their input order, like ``stable=True`` / ``kind='stable'``); -0.0 orders
before +0.0 (both frameworks treat them as equal); ``np_sort`` writes NaN as
the canonical quiet NaN (the reference qsort's ``hasnan`` behaviour).
"""
from __future__ import annotations

import numpy as np

import pyxss

_TORCH_NAMES = {
    "torch.float16": "float16", "torch.float32": "float32", "torch.float64": "float64",
    "torch.int16": "int16", "torch.int32": "int32", "torch.int64": "int64",
    "torch.uint16": "uint16", "torch.uint32": "uint32", "torch.uint64": "uint64",
}
_KV_KEYS = {"float32", "float64", "int32", "int64", "uint32", "uint64"}


def _torch():
    import torch
    return torch


def _dt(t) -> str:
    name = _TORCH_NAMES.get(str(t.dtype))
    if name is None:
        raise TypeError(f"unsupported dtype {t.dtype}")
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    return name


def _stream() -> int:
    return _torch().cuda.current_stream().cuda_stream


def sort(t, dim: int = -1, descending: bool = False):
    """(values, indices) of ``t`` sorted along its last dimension, like
    ``torch.sort(t, dim=-1, descending=descending, stable=True)``."""
    torch = _torch()
    dt = _dt(t)
    if dim not in (-1, t.dim() - 1):
        raise ValueError("only the last dimension is supported")
    x = t.contiguous()
    m = x.shape[-1] if x.dim() else 1
    rows = x.numel() // m if m else 0
    if x.numel() <= 1 or m <= 1:
        return x.clone(), torch.zeros_like(x, dtype=torch.int64)
    if rows == 1:
        idx = torch.empty(m, dtype=torch.int64, device=x.device)
        pyxss.gpu_argsort(dt, x.data_ptr(), idx.data_ptr(), m, True, descending,
                          stream=_stream())
        vals = x.reshape(-1).index_select(0, idx)
        return vals.view(x.shape), idx.view(x.shape)
    # one launch sequence for every row: segmented key-value sort
    keys = x.reshape(-1).clone()
    idx = torch.arange(m, dtype=torch.int64, device=x.device).repeat(rows)
    h_off = np.arange(0, rows * m + 1, m, dtype=np.uint64)
    d_off = torch.from_numpy(h_off.view(np.int64)).to(x.device)
    pyxss.gpu_segmented_sort(dt, "uint64", keys.data_ptr(), idx.data_ptr(), d_off.data_ptr(),
                             h_off, rows, True, descending, stream=_stream())
    return keys.view(x.shape), idx.view(x.shape)


def argsort(t, dim: int = -1, descending: bool = False):
    """Indices that sort ``t`` along its last dimension (stable)."""
    return sort(t, dim, descending)[1]


def kthvalue(t, k: int):
    """(value, index) of the k-th smallest element (k counts from 1) of a 1-D
    tensor, like ``torch.kthvalue``."""
    torch = _torch()
    dt = _dt(t)
    x = t.contiguous().reshape(-1)
    n = x.numel()
    if not 1 <= k <= n:
        raise ValueError("k out of range")
    arg = torch.empty(n, dtype=torch.int64, device=x.device)
    pyxss.gpu_argselect(dt, x.data_ptr(), arg.data_ptr(), k - 1, n, True, stream=_stream())
    i = arg[k - 1]
    return x[i], i


def topk(t, k: int, largest: bool = True):
    """(values, indices) of the k largest (or smallest) elements of a 1-D
    tensor in sorted order, like ``torch.topk(t, k, largest, sorted=True)``."""
    torch = _torch()
    dt = _dt(t)
    x = t.contiguous().reshape(-1)
    n = x.numel()
    if not 0 <= k <= n:
        raise ValueError("k out of range")
    if k == 0:
        return x[:0].clone(), torch.empty(0, dtype=torch.int64, device=x.device)
    if dt in _KV_KEYS and n > 1:
        keys = x.clone()
        idx = torch.arange(n, dtype=torch.int64, device=x.device)
        pyxss.gpu_keyvalue_partial_sort(dt, "uint64", keys.data_ptr(), idx.data_ptr(), k, n,
                                        True, largest, stream=_stream())
        return keys[:k].clone(), idx[:k].clone()
    vals, idx = sort(x, descending=largest)
    return vals[:k].clone(), idx[:k].clone()


# ---- NumPy-style, host arrays ------------------------------------------------------
def np_sort(a: np.ndarray) -> np.ndarray:
    """Sorted copy of a 1-D array (``np.sort``)."""
    b = np.ascontiguousarray(a).copy()
    if b.size > 1:
        pyxss.qsort(b, hasnan=True)
    return b


def np_argsort(a: np.ndarray) -> np.ndarray:
    """Stable sorting permutation of a 1-D array (``np.argsort(kind='stable')``)."""
    a = np.ascontiguousarray(a)
    if a.size <= 1:
        return np.zeros(a.size, dtype=np.int64)
    return pyxss.argsort(a, hasnan=True).astype(np.int64)


def np_partition(a: np.ndarray, kth: int) -> np.ndarray:
    """Copy of a 1-D array with the kth element in sorted position, smaller
    elements before it and larger after (``np.partition``)."""
    b = np.ascontiguousarray(a).copy()
    if not 0 <= kth < max(b.size, 1):
        raise ValueError("kth out of range")
    if b.size > 1:
        pyxss.qselect(b, kth, hasnan=True)
    return b


def np_argpartition(a: np.ndarray, kth: int) -> np.ndarray:
    """Index permutation that partitions a 1-D array around kth (``np.argpartition``)."""
    a = np.ascontiguousarray(a)
    if not 0 <= kth < max(a.size, 1):
        raise ValueError("kth out of range")
    if a.size <= 1:
        return np.zeros(a.size, dtype=np.int64)
    return pyxss.argselect(a, kth, hasnan=True).astype(np.int64)

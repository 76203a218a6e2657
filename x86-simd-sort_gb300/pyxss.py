"""ctypes binding of libxss_gb300.so, mirroring x86simdsort's API.

Host-array functions take NumPy arrays and work in place, with the reference's
names, argument order and defaults (lib/x86simdsort.h:15-70): ``qsort``,
``qselect``, ``partial_qsort``, ``argsort``, ``argselect``, ``keyvalue_qsort``,
``keyvalue_select``, ``keyvalue_partial_sort``.  Device functions (``gpu_*``)
take raw device pointers (ints) plus a dtype name, or torch CUDA tensors, and
run asynchronously on the given stream.

There is no CPU fallback: if the shared library is missing, importing works
but every call raises ``RuntimeError``.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
# XSS_LIB points at another build of the same library (e.g. a tuning variant)
LIB_PATH = os.environ.get("XSS_LIB") or os.path.join(PKG_DIR, "libxss_gb300.so")

DTYPES = {
    "uint16": 0, "int16": 1, "float16": 2,
    "uint32": 3, "int32": 4, "float32": 5,
    "uint64": 6, "int64": 7, "float64": 8,
}
KEY_BYTES = {0: 2, 1: 2, 2: 2, 3: 4, 4: 4, 5: 4, 6: 8, 7: 8, 8: 8}
OPS = {"qsort": 0, "qselect": 1, "partial_qsort": 2, "argsort": 3, "argselect": 4,
       "keyvalue_qsort": 5, "keyvalue_select": 6, "keyvalue_partial_sort": 7}
STATUS = {0: "ok", 1: "EINVAL", 2: "ENOMEM", 3: "ETIMEOUT", 4: "ECUDA",
          5: "EUNSUPPORTED", 6: "ETOOBIG"}


class XssError(RuntimeError):
    def __init__(self, code: int, what: str):
        super().__init__(f"{what}: {STATUS.get(code, code)}")
        self.code = code


_lib = None

_P = ctypes.c_void_p
_Z = ctypes.c_size_t
_I = ctypes.c_int
_SIGS = {
    "xss_strerror": (ctypes.c_char_p, [_I]),
    "xss_version": (ctypes.c_char_p, []),
    "xss_gpu_workspace_size": (_Z, [_I, _I, _I, _Z, _Z]),
    "xss_gpu_stream_status": (_I, [_P]),
    "xss_release_cached": (_I, []),
    "xss_gpu_qsort": (_I, [_I, _P, _Z, _I, _I, _P, _Z, _P]),
    "xss_gpu_qselect": (_I, [_I, _P, _Z, _Z, _I, _I, _P, _Z, _P]),
    "xss_gpu_partial_qsort": (_I, [_I, _P, _Z, _Z, _I, _I, _P, _Z, _P]),
    "xss_gpu_argsort": (_I, [_I, _P, _P, _Z, _I, _I, _P, _Z, _P]),
    "xss_gpu_argselect": (_I, [_I, _P, _P, _Z, _Z, _I, _P, _Z, _P]),
    "xss_gpu_keyvalue_qsort": (_I, [_I, _I, _P, _P, _Z, _I, _I, _P, _Z, _P]),
    "xss_gpu_keyvalue_select": (_I, [_I, _I, _P, _P, _Z, _Z, _I, _I, _P, _Z, _P]),
    "xss_gpu_keyvalue_partial_sort": (_I, [_I, _I, _P, _P, _Z, _Z, _I, _I, _P, _Z, _P]),
    "xss_gpu_segmented_sort": (_I, [_I, _I, _P, _P, _P, _P, _Z, _I, _I, _P, _Z, _P]),
    "xss_gpu_segmented_workspace_size": (_Z, [_I, _I, _P, _Z]),
    "xss_gpu_segmented_topk": (_I, [_I, _I, _P, _P, _P, _P, _Z, _Z, _I, _I, _P, _Z, _P]),
    "xss_qsort": (_I, [_I, _P, _Z, _I, _I]),
    "xss_qselect": (_I, [_I, _P, _Z, _Z, _I, _I]),
    "xss_partial_qsort": (_I, [_I, _P, _Z, _Z, _I, _I]),
    "xss_argsort": (_I, [_I, _P, _P, _Z, _I, _I]),
    "xss_argselect": (_I, [_I, _P, _P, _Z, _Z, _I]),
    "xss_keyvalue_qsort": (_I, [_I, _I, _P, _P, _Z, _I, _I]),
    "xss_keyvalue_select": (_I, [_I, _I, _P, _P, _Z, _Z, _I, _I]),
    "xss_keyvalue_partial_sort": (_I, [_I, _I, _P, _P, _Z, _Z, _I, _I]),
    "xss_seg_plan_create": (_I, [ctypes.POINTER(_P), _I, _I, _P, _Z, _I, _I]),
    "xss_seg_plan_workspace_size": (_Z, [_P]),
    "xss_seg_plan_run": (_I, [_P, _P, _P, _P, _P, _Z, _P, _I]),
    "xss_seg_plan_destroy": (None, [_P]),
    "xss_gpu_segmented_sort_percall": (_I, [_I, _I, _P, _P, _P, _Z, _I, _I, _P]),
    "xss_gpu_object_qsort": (_I, [_P, _Z, _Z, _Z, _I, _I, _I, _P, _Z, _P]),
    "xss_gpu_object_workspace_size": (_Z, [_Z, _Z, _I]),
    "xss_prof_enable": (None, [_I]),
    "xss_prof_reset": (None, []),
    "xss_prof_read": (_I, [_I, ctypes.POINTER(ctypes.c_double),
                           ctypes.POINTER(ctypes.c_ulonglong)]),
    "xss_prof_launches": (ctypes.c_ulonglong, [_I]),
    "xss_prof_kind_name": (ctypes.c_char_p, [_I]),
}

PROF_KINDS = ["hist", "onesweep", "fixup", "small_sort", "sel_hist", "sel_find",
              "sel_collect", "sel_place", "seg_small", "seg_block", "seg_misc", "object",
              "merge", "count16"]


def prof_enable(on: bool) -> None:
    lib().xss_prof_enable(int(on))


def prof_reset() -> None:
    lib().xss_prof_reset()


def prof_read(kind: str):
    """(total event-timed ms, timed launches) for a kernel kind since prof_reset()."""
    ms = ctypes.c_double(0)
    cnt = ctypes.c_ulonglong(0)
    lib().xss_prof_read(PROF_KINDS.index(kind), ctypes.byref(ms), ctypes.byref(cnt))
    return ms.value, cnt.value


def prof_launches() -> int:
    """Total kernel launches by the library so far (all kinds)."""
    return sum(lib().xss_prof_launches(i) for i in range(len(PROF_KINDS)))


def lib() -> ctypes.CDLL:
    """Load libxss_gb300.so once; raise if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in _SIGS.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def dtype_id(dt) -> int:
    name = np.dtype(dt).name if not isinstance(dt, str) else dt
    if name not in DTYPES:
        raise TypeError(f"unsupported key type {name}")
    return DTYPES[name]


def check(rc: int, what: str) -> None:
    if rc != 0:
        raise XssError(rc, what)


def _ptr(a: np.ndarray) -> int:
    if not a.flags.c_contiguous:
        raise ValueError("array must be C-contiguous")
    return a.ctypes.data


# ---- host arrays (in place), reference names and defaults ---------------------
def qsort(arr: np.ndarray, hasnan: bool = False, descending: bool = False) -> None:
    check(lib().xss_qsort(dtype_id(arr.dtype), _ptr(arr), arr.size, int(hasnan),
                          int(descending)), "qsort")


def qselect(arr: np.ndarray, k: int, hasnan: bool = False, descending: bool = False) -> None:
    check(lib().xss_qselect(dtype_id(arr.dtype), _ptr(arr), k, arr.size, int(hasnan),
                            int(descending)), "qselect")


def partial_qsort(arr: np.ndarray, k: int, hasnan: bool = False,
                  descending: bool = False) -> None:
    check(lib().xss_partial_qsort(dtype_id(arr.dtype), _ptr(arr), k, arr.size, int(hasnan),
                                  int(descending)), "partial_qsort")


def argsort(arr: np.ndarray, hasnan: bool = False, descending: bool = False,
            out: np.ndarray = None) -> np.ndarray:
    """Indices that sort arr; into `out` (uint64, arr.size) when given, as the
    reference's argsort(T*, size_t* arg, ...) writes into the caller's array."""
    if out is None:
        out = np.empty(arr.size, dtype=np.uint64)
    assert out.dtype == np.uint64 and out.size == arr.size
    check(lib().xss_argsort(dtype_id(arr.dtype), _ptr(arr), _ptr(out), arr.size, int(hasnan),
                            int(descending)), "argsort")
    return out


def argselect(arr: np.ndarray, k: int, hasnan: bool = False,
              out: np.ndarray = None) -> np.ndarray:
    if out is None:
        out = np.empty(arr.size, dtype=np.uint64)
    assert out.dtype == np.uint64 and out.size == arr.size
    check(lib().xss_argselect(dtype_id(arr.dtype), _ptr(arr), _ptr(out), k, arr.size,
                              int(hasnan)), "argselect")
    return out


def keyvalue_qsort(keys: np.ndarray, vals: np.ndarray, hasnan: bool = False,
                   descending: bool = False) -> None:
    assert keys.size == vals.size
    check(lib().xss_keyvalue_qsort(dtype_id(keys.dtype), dtype_id(vals.dtype), _ptr(keys),
                                   _ptr(vals), keys.size, int(hasnan), int(descending)),
          "keyvalue_qsort")


def keyvalue_select(keys: np.ndarray, vals: np.ndarray, k: int, hasnan: bool = False,
                    descending: bool = False) -> None:
    assert keys.size == vals.size
    check(lib().xss_keyvalue_select(dtype_id(keys.dtype), dtype_id(vals.dtype), _ptr(keys),
                                    _ptr(vals), k, keys.size, int(hasnan), int(descending)),
          "keyvalue_select")


def keyvalue_partial_sort(keys: np.ndarray, vals: np.ndarray, k: int, hasnan: bool = False,
                          descending: bool = False) -> None:
    assert keys.size == vals.size
    check(lib().xss_keyvalue_partial_sort(dtype_id(keys.dtype), dtype_id(vals.dtype),
                                          _ptr(keys), _ptr(vals), k, keys.size, int(hasnan),
                                          int(descending)), "keyvalue_partial_sort")


# ---- device pointers ------------------------------------------------------------
def workspace_size(op: str, key_dtype, n: int, k: int = 0, val_dtype="uint64") -> int:
    return lib().xss_gpu_workspace_size(OPS[op], dtype_id(key_dtype), dtype_id(val_dtype), n, k)


def stream_status(stream: int = 0) -> None:
    check(lib().xss_gpu_stream_status(stream or None), "device status")


def release_cached() -> None:
    """Free the library's cached device buffers on the current device (every
    stream's workspace, this thread's host-pointer staging and pipeline
    buffers)."""
    check(lib().xss_release_cached(), "release cached")


def gpu_qsort(dt, d_arr: int, n: int, hasnan=False, descending=False, ws=0, ws_bytes=0,
              stream=0) -> None:
    check(lib().xss_gpu_qsort(dtype_id(dt), d_arr, n, int(hasnan), int(descending),
                              ws or None, ws_bytes, stream or None), "gpu_qsort")


def gpu_qselect(dt, d_arr, k, n, hasnan=False, descending=False, ws=0, ws_bytes=0, stream=0):
    check(lib().xss_gpu_qselect(dtype_id(dt), d_arr, k, n, int(hasnan), int(descending),
                                ws or None, ws_bytes, stream or None), "gpu_qselect")


def gpu_partial_qsort(dt, d_arr, k, n, hasnan=False, descending=False, ws=0, ws_bytes=0,
                      stream=0):
    check(lib().xss_gpu_partial_qsort(dtype_id(dt), d_arr, k, n, int(hasnan), int(descending),
                                      ws or None, ws_bytes, stream or None), "gpu_partial_qsort")


def gpu_argsort(dt, d_arr, d_arg, n, hasnan=False, descending=False, ws=0, ws_bytes=0,
                stream=0):
    check(lib().xss_gpu_argsort(dtype_id(dt), d_arr, d_arg, n, int(hasnan), int(descending),
                                ws or None, ws_bytes, stream or None), "gpu_argsort")


def gpu_argselect(dt, d_arr, d_arg, k, n, hasnan=False, ws=0, ws_bytes=0, stream=0):
    check(lib().xss_gpu_argselect(dtype_id(dt), d_arr, d_arg, k, n, int(hasnan), ws or None,
                                  ws_bytes, stream or None), "gpu_argselect")


def gpu_keyvalue_qsort(kdt, vdt, d_keys, d_vals, n, hasnan=False, descending=False, ws=0,
                       ws_bytes=0, stream=0):
    check(lib().xss_gpu_keyvalue_qsort(dtype_id(kdt), dtype_id(vdt), d_keys, d_vals, n,
                                       int(hasnan), int(descending), ws or None, ws_bytes,
                                       stream or None), "gpu_keyvalue_qsort")


def gpu_keyvalue_select(kdt, vdt, d_keys, d_vals, k, n, hasnan=False, descending=False, ws=0,
                        ws_bytes=0, stream=0):
    check(lib().xss_gpu_keyvalue_select(dtype_id(kdt), dtype_id(vdt), d_keys, d_vals, k, n,
                                        int(hasnan), int(descending), ws or None, ws_bytes,
                                        stream or None), "gpu_keyvalue_select")


def gpu_keyvalue_partial_sort(kdt, vdt, d_keys, d_vals, k, n, hasnan=False, descending=False,
                              ws=0, ws_bytes=0, stream=0):
    check(lib().xss_gpu_keyvalue_partial_sort(dtype_id(kdt), dtype_id(vdt), d_keys, d_vals, k,
                                              n, int(hasnan), int(descending), ws or None,
                                              ws_bytes, stream or None),
          "gpu_keyvalue_partial_sort")


def gpu_segmented_sort(kdt, vdt, d_keys, d_vals, d_offsets, h_offsets: np.ndarray,
                       num_segments, hasnan=False, descending=False, ws=0, ws_bytes=0,
                       stream=0):
    hp = _ptr(h_offsets) if h_offsets is not None else None
    check(lib().xss_gpu_segmented_sort(dtype_id(kdt), dtype_id(vdt) if vdt else -1, d_keys,
                                       d_vals or None, d_offsets or None, hp, num_segments,
                                       int(hasnan), int(descending), ws or None, ws_bytes,
                                       stream or None), "gpu_segmented_sort")


def gpu_segmented_topk(kdt, vdt, d_keys, d_vals, d_offsets, h_offsets: np.ndarray,
                       num_segments, k, hasnan=False, descending=False, ws=0, ws_bytes=0,
                       stream=0):
    """Each segment's min(k, len) smallest keys (largest when descending), in
    order, at its front (xss_gpu_segmented_topk)."""
    hp = _ptr(h_offsets) if h_offsets is not None else None
    check(lib().xss_gpu_segmented_topk(dtype_id(kdt), dtype_id(vdt) if vdt else -1, d_keys,
                                       d_vals or None, d_offsets or None, hp, num_segments, k,
                                       int(hasnan), int(descending), ws or None, ws_bytes,
                                       stream or None), "gpu_segmented_topk")


def segmented_workspace_size(kdt, vdt, h_offsets: np.ndarray) -> int:
    return lib().xss_gpu_segmented_workspace_size(dtype_id(kdt), dtype_id(vdt) if vdt else -1,
                                                  _ptr(h_offsets), h_offsets.size - 1)


def gpu_segmented_sort_percall(kdt, vdt, d_keys, d_vals, h_offsets: np.ndarray, hasnan=False,
                               descending=False, stream=0):
    check(lib().xss_gpu_segmented_sort_percall(dtype_id(kdt), dtype_id(vdt) if vdt else -1,
                                               d_keys, d_vals or None, _ptr(h_offsets),
                                               h_offsets.size - 1, int(hasnan), int(descending),
                                               stream or None), "segmented_sort_percall")


def gpu_object_qsort(d_recs, n, rec_bytes, key_offset, key_dtype, hasnan=False,
                     descending=False, ws=0, ws_bytes=0, stream=0):
    """Sort n records of rec_bytes bytes in device memory by the key at key_offset."""
    check(lib().xss_gpu_object_qsort(d_recs, n, rec_bytes, key_offset, dtype_id(key_dtype),
                                     int(hasnan), int(descending), ws or None, ws_bytes,
                                     stream or None), "gpu_object_qsort")


def object_workspace_size(n, rec_bytes, key_dtype) -> int:
    return lib().xss_gpu_object_workspace_size(n, rec_bytes, dtype_id(key_dtype))


class SegPlan:
    """A reusable segmented-sort plan (xss_seg_plan_*) for one offsets layout."""

    def __init__(self, kdt, vdt, h_offsets: np.ndarray, hasnan=False, descending=False):
        self._h = ctypes.c_void_p()
        self._off = np.ascontiguousarray(h_offsets, dtype=np.uint64)
        check(lib().xss_seg_plan_create(ctypes.byref(self._h), dtype_id(kdt),
                                        dtype_id(vdt) if vdt else -1, _ptr(self._off),
                                        self._off.size - 1, int(hasnan), int(descending)),
              "seg_plan_create")

    @property
    def workspace_size(self) -> int:
        return lib().xss_seg_plan_workspace_size(self._h)

    def run(self, d_keys, d_vals, d_offsets, ws, ws_bytes, stream=0, use_graph=True):
        check(lib().xss_seg_plan_run(self._h, d_keys, d_vals or None, d_offsets, ws, ws_bytes,
                                     stream or None, int(use_graph)), "seg_plan_run")

    def close(self):
        if self._h:
            lib().xss_seg_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---- serving loop -----------------------------------------------------------------
class ServeRequest(ctypes.Structure):
    _fields_ = [("op", _I), ("key_dtype", _I), ("val_dtype", _I), ("keys_in", _P),
                ("keys_out", _P), ("vals_in", _P), ("vals_out", _P), ("arg_out", _P),
                ("n", _Z), ("k", _Z), ("hasnan", _I), ("descending", _I)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("device", _I), ("hbm_budget_bytes", _Z), ("streams", _I), ("small_max", _Z),
                ("max_batch", _Z), ("max_queue", _Z)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("shed", ctypes.c_uint64),
                ("completed", ctypes.c_uint64), ("failed", ctypes.c_uint64),
                ("batches", ctypes.c_uint64), ("batched_requests", ctypes.c_uint64),
                ("keys", ctypes.c_double), ("wall_s", ctypes.c_double),
                ("p50_us", ctypes.c_double), ("p99_us", ctypes.c_double),
                ("max_us", ctypes.c_double), ("pool_bytes", _Z)]


_SERVER_SIGS = {
    "xss_server_create": (_I, [ctypes.POINTER(_P), ctypes.POINTER(ServerConfig)]),
    "xss_server_submit": (_I, [_P, ctypes.POINTER(ServeRequest), ctypes.POINTER(ctypes.c_uint64)]),
    "xss_server_wait": (_I, [_P, ctypes.c_uint64, ctypes.POINTER(_I)]),
    "xss_server_poll": (_I, [_P, ctypes.c_uint64, ctypes.POINTER(_I)]),
    "xss_server_get_stats": (_I, [_P, ctypes.POINTER(ServerStats)]),
    "xss_server_reset_stats": (_I, [_P]),
    "xss_server_destroy": (None, [_P, _I]),
}


class Server:
    """xss_server_*: submit requests on (preferably pinned) host buffers."""

    def __init__(self, device=0, hbm_budget_bytes=0, streams=0, small_max=0, max_batch=0,
                 max_queue=0):
        L = lib()
        for name, (res, args) in _SERVER_SIGS.items():
            f = getattr(L, name)
            f.restype, f.argtypes = res, args
        self._L = L
        self._h = _P()
        cfg = ServerConfig(device, hbm_budget_bytes, streams, small_max, max_batch, max_queue)
        check(L.xss_server_create(ctypes.byref(self._h), ctypes.byref(cfg)), "server_create")

    def submit(self, op, key_dtype, keys_in, keys_out=None, n=None, k=0, vals_in=None,
               vals_out=None, val_dtype="uint64", arg_out=None, hasnan=False, descending=False):
        """Returns a ticket, or None when the server refused the request (shed)."""
        r = ServeRequest(OPS[op], dtype_id(key_dtype), dtype_id(val_dtype), keys_in,
                         keys_out or keys_in, vals_in, vals_out or vals_in, arg_out, n, k,
                         int(hasnan), int(descending))
        t = ctypes.c_uint64(0)
        rc = self._L.xss_server_submit(self._h, ctypes.byref(r), ctypes.byref(t))
        if rc == 7:
            return None
        check(rc, "server_submit")
        return t.value

    def wait(self, ticket) -> int:
        st = _I(0)
        check(self._L.xss_server_wait(self._h, ticket, ctypes.byref(st)), "server_wait")
        return st.value

    def poll(self, ticket):
        """Request status code, or None while it is pending."""
        st = _I(0)
        rc = self._L.xss_server_poll(self._h, ticket, ctypes.byref(st))
        return None if rc == 8 else st.value

    def stats(self) -> dict:
        s = ServerStats()
        check(self._L.xss_server_get_stats(self._h, ctypes.byref(s)), "server_stats")
        return {name: getattr(s, name) for name, _ in ServerStats._fields_}

    def reset_stats(self):
        self._L.xss_server_reset_stats(self._h)

    def close(self, drain=True):
        if self._h:
            self._L.xss_server_destroy(self._h, int(drain))
            self._h = _P()

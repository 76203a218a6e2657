"""ctypes access to the CPU oracle (TEST INFRASTRUCTURE ONLY).

``oracle()`` is the portable C++ restatement (oracle/xss_oracle.cpp) of the
reference's scalar path; ``reference()`` is the reference library itself,
compiled from its sources into oracle/_ref/ where the host can build it
(x86-64), else None.  Both expose the same functions (prefixes xo_ / xr_).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "libxss_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libxss_refshim.so")
# the reference's source tree, when given (build_reference argument or this variable)
REF_SRC = os.environ.get("XSS_REFERENCE_SRC")

_P, _Z, _I = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
_FUNCS = {
    "qsort": [_I, _P, _Z, _I, _I],
    "qselect": [_I, _P, _Z, _Z, _I, _I],
    "partial_qsort": [_I, _P, _Z, _Z, _I, _I],
    "argsort": [_I, _P, _P, _Z, _I, _I],
    "argselect": [_I, _P, _P, _Z, _Z, _I],
    "keyvalue_qsort": [_I, _I, _P, _P, _Z, _I, _I],
    "keyvalue_select": [_I, _I, _P, _P, _Z, _Z, _I, _I],
    "keyvalue_partial_sort": [_I, _I, _P, _P, _Z, _Z, _I, _I],
}
_ORACLE_EXTRA = {
    "compare": [_I, _I, _P, _P],
    "max_threads": [],
    "qsort_mt": [_I, _P, _Z, _I, _I, _I],
    "argsort_mt": [_I, _P, _P, _Z, _I, _I, _I],
    "keyvalue_qsort_mt": [_I, _I, _P, _P, _Z, _I, _I, _I],
}


class _Lib:
    def __init__(self, path: str, prefix: str, extra: dict):
        self._l = ctypes.CDLL(path)
        for name, args in {**_FUNCS, **extra}.items():
            f = getattr(self._l, prefix + name)
            f.restype = _I
            f.argtypes = args
            setattr(self, name, f)


_oracle = None
_ref = None


def build_oracle() -> str:
    """Compile the portable oracle (make -C oracle oracle)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    return ORACLE_SO


def build_reference(src: str | None = None) -> str | None:
    """Compile the reference from its sources (``src``, else $XSS_REFERENCE_SRC)
    into oracle/_ref when possible; None where no source tree is given or the
    host cannot build it (the reference's SIMD paths need x86-64)."""
    src = src or REF_SRC
    if not src or not os.path.isdir(src) or os.uname().machine not in ("x86_64", "AMD64"):
        return None
    r = subprocess.run(["make", "-s", "-j5", "-C", HERE, "ref", f"REF={src}"])
    return REF_SO if r.returncode == 0 and os.path.exists(REF_SO) else None


def oracle() -> _Lib:
    global _oracle
    if _oracle is None:
        if not os.path.exists(ORACLE_SO):
            build_oracle()
        _oracle = _Lib(ORACLE_SO, "xo_", _ORACLE_EXTRA)
    return _oracle


def reference() -> _Lib | None:
    """The reference library built from source, or None where it cannot load."""
    global _ref
    if _ref is None and os.path.exists(REF_SO):
        try:
            _ref = _Lib(REF_SO, "xr_", {})
        except OSError:
            return None
    return _ref

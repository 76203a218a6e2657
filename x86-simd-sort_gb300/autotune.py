"""Offline autotuner for the onesweep radix pass.

Each (key width, value width) class of the pass kernel has a tuning line
``XSS_CFG_<class> BLOCK, ITEMS, MINB, LB, RANK, PERSIST, DPT`` for large
arrays and ``XSS_CFGM_<class>`` for arrays up to ``XSS_MID_N`` keys (class
names ending in ``_MID``; meaning of each field: the comment above ``CfgT``
in ``csrc/xss_onesweep.cuh``).  This
tool builds one library per candidate line (the candidate is pre-included as
a header, so the sources stay untouched), times each on the GPU with CUDA
events on full-size uniform inputs, checks every result, and writes the
fastest line per class to a header::

    python x86-simd-sort_gb300/autotune.py --classes K32,K64V64,K32_MID --out xss_tuning.h

Copy the written header to ``csrc/xss_tuning.h``; ``xss_onesweep.cuh``
includes it when present, so the next build uses the tuned lines.  Timing
runs in a child process per candidate (each loads its own library through
``XSS_LIB``).  Candidate lists are per class; ``--candidates`` replaces them
(``K32=512,16,2,16,0,1,1;K32=...``).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys
import time

PKG = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, PKG)
import build as _build  # noqa: E402

TUNE_DIR = os.path.join(PKG, "_build", "tune")

# class -> (key dtype, value dtype or None) used to time it
CLASSES = {
    "K16": ("uint16", None),
    "K32": ("uint32", None),
    "K64": ("uint64", None),
    "K32V32": ("uint32", "uint32"),
    "K64V64": ("uint64", "uint64"),
    "DEFAULT": ("uint64", "uint32"),
}

# Candidate lines (BLOCK, ITEMS, MINB, LB, RANK, PERSIST, DPT).  They stay
# within 64K registers per SM at MINB CTAs and the 227 KB shared-memory cap.
CANDIDATES = {
    "K16": ["320,20,3,16,2,1,0", "512,16,2,16,2,1,0"],
    "K32": ["320,20,3,8,2,1,0", "320,20,3,16,2,1,0", "512,16,2,8,2,1,0", "384,16,3,8,2,1,0",
            "256,24,3,8,2,1,0", "256,16,4,8,2,1,0", "320,16,4,8,2,1,0"],
    "K64": ["512,16,1,16,2,1,1", "512,20,1,16,2,1,1", "512,24,1,16,2,1,1", "768,16,1,16,2,1,1"],
    "K32V32": ["512,14,1,16,2,1,1", "512,20,1,16,2,1,1", "768,14,1,16,2,1,1"],
    "K64V64": ["512,11,1,8,2,1,1", "512,12,1,8,2,1,1", "640,10,1,8,2,1,1", "768,8,1,8,2,1,1",
               "384,16,1,8,2,1,1", "512,12,1,16,2,1,1"],
    "DEFAULT": ["512,14,1,8,2,1,1", "512,16,1,8,2,1,1", "640,12,1,8,2,1,1", "768,10,1,8,2,1,1"],
    # mid-size arrays: several CTAs per SM (tile or resident form)
    "K16_MID": ["512,16,2,16,2,1,0", "256,16,3,16,2,1,0"],
    "K32_MID": ["512,16,2,16,2,1,0", "256,16,3,16,2,1,0", "256,8,4,16,2,1,0"],
    "K64_MID": ["512,8,2,16,2,1,1", "256,16,2,16,2,1,0"],
    "K32V32_MID": ["512,10,2,16,2,0,0", "512,10,2,16,2,1,1"],
    "K64V64_MID": ["512,6,2,16,2,0,1", "256,12,2,16,2,0,0"],
    "DEFAULT_MID": ["512,6,2,16,2,0,1", "256,8,3,16,2,0,0"],
}


def _base(cls: str):
    """(width class, macro name, is mid-size) of a class name."""
    mid = cls.endswith("_MID")
    base = cls[:-4] if mid else cls
    return base, ("XSS_CFGM_" if mid else "XSS_CFG_") + base, mid


def _run(cmd, **kw):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, **kw)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout[-2000:])
    return r.stdout


def build_variant(cls: str, line: str, common_objs: list) -> str:
    """Compile the radix unit with one candidate line pre-included; link a library."""
    tag = f"{cls}_{line.replace(',', '_')}"
    os.makedirs(TUNE_DIR, exist_ok=True)
    hdr = os.path.join(TUNE_DIR, f"cfg_{tag}.h")
    with open(hdr, "w") as f:
        f.write(f"#define {_base(cls)[1]} {line}\n")
    obj = os.path.join(TUNE_DIR, f"radix_{tag}.o")
    _run([_build.NVCC] + _build.ARCH + _build.NVCC_FLAGS +
         ["--pre-include", hdr, "-c", os.path.join(_build.CSRC, "xss_radix.cu"), "-o", obj])
    so = os.path.join(TUNE_DIR, f"lib_{tag}.so")
    _run([_build.NVCC] + _build.ARCH + ["-shared", "-o", so, obj] + common_objs +
         ["-cudart", "shared"])
    return so


def build_common() -> list:
    """Objects of every unit except the radix one (built once, shared by all variants)."""
    _build.build()
    objs = []
    for name in sorted(os.listdir(_build.BUILD)):
        if name.endswith(".o") and not name.startswith("xss_radix"):
            objs.append(os.path.join(_build.BUILD, name))
    return objs


def measure(cls: str, n: int, reps: int) -> dict:
    """Child-process side: time the class's sort with the library in XSS_LIB."""
    import torch
    import pyxss
    kdt, vdt = CLASSES[_base(cls)[0]]
    tdt = {"uint16": torch.int16, "uint32": torch.int32, "uint64": torch.int64}
    kb = {"uint16": 2, "uint32": 4, "uint64": 8}[kdt]
    g = torch.Generator(device="cuda").manual_seed(7)
    k0 = torch.randint(0, 256, (n * kb,), dtype=torch.uint8, device="cuda",
                       generator=g).view(tdt[kdt])
    keys = k0.clone()
    vals = None
    if vdt is not None:
        vals = torch.arange(n, dtype=tdt[vdt], device="cuda")
    stream = torch.cuda.current_stream()
    times = []
    for r in range(reps + 2):
        keys.copy_(k0)
        if vals is not None:
            vals.copy_(torch.arange(n, dtype=vals.dtype, device="cuda"))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        if vals is None:
            pyxss.gpu_qsort(kdt, keys.data_ptr(), n, stream=stream.cuda_stream)
        else:
            pyxss.gpu_keyvalue_qsort(kdt, vdt, keys.data_ptr(), vals.data_ptr(), n,
                                     stream=stream.cuda_stream)
        e1.record(stream)
        e1.synchronize()
        if r >= 2:
            times.append(e0.elapsed_time(e1))
    pyxss.stream_status(stream.cuda_stream)
    # checks: unsigned order of the keys (compared as 32-bit halves, since
    # torch compares 64-bit integers signed); values a permutation carrying
    # their keys
    w = keys.to(torch.int64)
    if kb == 8:
        hi, lo = (w >> 32) & 0xFFFFFFFF, w & 0xFFFFFFFF
        okk = bool(((hi[1:] > hi[:-1]) | ((hi[1:] == hi[:-1]) & (lo[1:] >= lo[:-1]))).all())
    else:
        w = w & ((1 << (8 * kb)) - 1)
        okk = bool((w[1:] >= w[:-1]).all())
    okv = True
    if vals is not None:
        idx = vals.to(torch.int64)
        seen = torch.zeros(n, dtype=torch.int32, device="cuda")
        seen.index_add_(0, idx, torch.ones(n, dtype=torch.int32, device="cuda"))
        okv = bool((seen == 1).all()) and bool((k0[idx] == keys).all())
    times.sort()
    return {"ms": times[len(times) // 2], "ok": okk and okv}


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--classes", default="K32,K64V64")
    ap.add_argument("--candidates", default="", help="CLASS=line;CLASS=line overrides")
    ap.add_argument("--n", type=int, default=1 << 28, help="keys for large-array classes")
    ap.add_argument("--n-mid", type=int, default=1 << 21, help="keys for _MID classes")
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--out", default=os.path.join(PKG, "_build", "xss_tuning.h"))
    ap.add_argument("--measure", default="", help=argparse.SUPPRESS)
    args = ap.parse_args()

    if args.measure:
        print(json.dumps(measure(args.measure, args.n, args.reps)))
        return

    classes = [c for c in args.classes.split(",") if c]
    cands = {c: list(CANDIDATES[c]) for c in classes}
    if args.candidates:
        cands = {}
        for item in args.candidates.split(";"):
            c, line = item.split("=", 1)
            cands.setdefault(c, []).append(line)
    os.makedirs(TUNE_DIR, exist_ok=True)
    common = build_common()
    jobs = [(c, line) for c, lines in cands.items() for line in lines]
    t0 = time.time()
    with cf.ThreadPoolExecutor(min(16, os.cpu_count() or 4)) as ex:
        libs = list(ex.map(lambda j: build_variant(j[0], j[1], common), jobs))
    print(f"built {len(libs)} variants in {time.time() - t0:.0f} s", flush=True)

    results = {}
    for (c, line), so in zip(jobs, libs):
        env = dict(os.environ, XSS_LIB=so)
        mid = _base(c)[2]
        r = subprocess.run([sys.executable, os.path.abspath(__file__), "--measure", c,
                            "--n", str(args.n_mid if mid else args.n),
                            "--reps", str(args.reps * 4 if mid else args.reps)],
                           env=env, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
        try:
            res = json.loads(r.stdout.strip().splitlines()[-1])
        except (ValueError, IndexError):
            res = {"ms": float("inf"), "ok": False, "error": r.stdout[-500:]}
        results.setdefault(c, []).append((line, res))
        print(f"{c:8s} {line:22s} {res['ms']:9.3f} ms  ok={res['ok']}", flush=True)

    with open(args.out, "w") as f:
        f.write("// xss_tuning.h -- onesweep pass lines chosen by autotune.py "
                f"(n = {args.n}, _MID classes n = {args.n_mid}; uniform keys; median time).\n")
        f.write("// Each line: BLOCK, ITEMS, MINB, LB, RANK, PERSIST, DPT.\n#pragma once\n")
        for c, rs in results.items():
            good = [(line, r) for line, r in rs if r["ok"]]
            if not good:
                continue
            best, br = min(good, key=lambda x: x[1]["ms"])
            f.write("\n// " + c + ": " + "; ".join(
                f"{line} {r['ms']:.3f} ms" for line, r in rs) + "\n")
            macro = _base(c)[1]
            f.write(f"#ifndef {macro}\n#define {macro} {best.replace(',', ', ')}\n#endif\n")
    print("wrote", args.out)


if __name__ == "__main__":
    main()

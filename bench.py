"""Benchmark of the GB300 sort/select library (one JSON line on stdout).

python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

Default workload: keyvalue_qsort of 2^28 int64 keys (uniform over the full
range) carrying uint64 values = original index, ascending -- the key-value
half of the reference's 2^28 configuration.  A step is one sort of the whole
array; the input is restored from a pristine device copy before every step,
outside the timed events (as the reference's benchmarks restore outside
PauseTiming, benchmarks/bench-qsort.hpp:31-36).  Inputs (4 GiB) are far larger
than L2, so no flush is needed between steps.

`value` is device-resident throughput (Gkeys/s, CUDA events on the launching
stream); `e2e` is the same sort through the host-pointer C ABI
(xss_keyvalue_qsort) from pinned host buffers, copies included; `roofline`
covers the dominant kernel (one onesweep radix pass) with its algorithmic
bytes per launch; `cpu_baseline` times the CPU oracle port (or the reference
library where it builds) on a bounded sample of the same workload.

Several ranks (torchrun) run independent replicas: a single array does not
shard without an all-to-all exchange, so each GPU sorts its own array and
`value` is the sum over ranks of keys sorted per unit of the slowest rank's
time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "x86-simd-sort_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, ROOT)


# ---------------------------------------------------------------------------
def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# dominant kernel at the workload's full size: one ncu capture of a smaller case
# scaled by the keys per launch (the int64 -> uint64 pass captured at 2^25
# keys x8; the float32 passes captured at 2^26 keys, their mean x4).
TRAFFIC = {"keyvalue_qsort": 8245616640, "qsort_f32": 1989168640}


def _traffic(workload, n, n_full):
    return TRAFFIC.get(workload) if n == n_full else None


class Clocks:
    """nvidia-smi samples (SM clock, throttle reasons) during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.rows = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(index), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) == 6:
                self.rows.append(parts)

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = [r for r in self.rows if r[0].isdigit()]
        if not rows:
            return None
        sm = [int(r[0]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[2 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][1]),
                "reasons": reasons, "samples": len(rows)}


# ---------------------------------------------------------------------------
class Workload:
    """One device-resident sort/select workload."""

    dominant = "onesweep"

    def __init__(self, torch, xss, n, stream):
        self.torch, self.xss, self.n, self.stream = torch, xss, n, stream
        self._pinned = []

    def pinned(self, nbytes: int, dtype) -> np.ndarray:
        """Pinned host buffer viewed as `dtype`; the tensor that owns the memory is
        kept alive with the workload (a dropped owner returns its block to torch's
        host allocator, and copies from it then ran at half speed)."""
        t = self.torch.empty(nbytes, dtype=self.torch.uint8, pin_memory=True)
        self._pinned.append(t)
        return t.numpy().view(dtype)

    def release(self):
        """Drop the workload's device and pinned buffers (several workloads run
        one after another in the default bench)."""
        plan = getattr(self, "plan", None)
        if plan is not None:
            plan.close()
        for k in list(vars(self)):
            v = getattr(self, k)
            if k == "plan" or k == "_pinned" or isinstance(v, np.ndarray) or \
                    (self.torch is not None and isinstance(v, self.torch.Tensor)):
                if k not in ("sizes", "off"):
                    setattr(self, k, None)


class KeyValueSort(Workload):
    name = "keyvalue_qsort"
    kdt, vdt, kb, vb = "int64", "uint64", 8, 8

    def describe(self):
        return {"workload": f"keyvalue_qsort int64->uint64 n=2^{self.n.bit_length() - 1} "
                            "uniform full-range keys, values=index, ascending",
                "n": self.n, "l2": "inputs (4 GiB) larger than L2; input restored per step"}

    def setup(self):
        t, n = self.torch, self.n
        g = t.Generator(device="cuda").manual_seed(1)
        self.k0 = t.randint(0, 256, (n * 8,), dtype=t.uint8, device="cuda",
                            generator=g).view(t.int64)
        self.v0 = t.arange(n, dtype=t.int64, device="cuda")
        self.k = t.empty_like(self.k0)
        self.v = t.empty_like(self.v0)
        self.wsb = self.xss.workspace_size("keyvalue_qsort", self.kdt, n, val_dtype=self.vdt)
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def restore(self):
        self.k.copy_(self.k0)
        self.v.copy_(self.v0)

    def run(self):
        self.xss.gpu_keyvalue_qsort(self.kdt, self.vdt, self.k.data_ptr(), self.v.data_ptr(),
                                    self.n, False, False, self.ws.data_ptr(), self.wsb,
                                    self.stream.cuda_stream)

    def check(self):
        t = self.torch
        k, v = self.k, self.v
        ok = bool((k[1:] >= k[:-1]).all())
        ok &= bool((self.k0[v] == k).all())
        cnt = t.zeros(self.n, dtype=t.int32, device="cuda")
        cnt.index_add_(0, v, t.ones(self.n, dtype=t.int32, device="cuda"))
        ok &= bool((cnt == 1).all())
        return ok

    def passes(self):
        return self.kb

    def bytes_per_pass(self):           # read + write of key and value
        return 2 * self.n * (self.kb + self.vb)

    def bytes_model(self):              # fixed model: n(kb + 2P(kb+vb))
        return self.n * (self.kb + 2 * self.passes() * (self.kb + self.vb))

    # host-pointer (e2e) path
    def host_setup(self):
        t = self.torch
        self.hk0 = self.k0.cpu().numpy()
        self.hv0 = self.v0.cpu().numpy().view(np.uint64)
        self.hk = self.pinned(self.n * 8, np.int64)
        self.hv = self.pinned(self.n * 8, np.uint64)

    def host_restore(self):
        np.copyto(self.hk, self.hk0)
        np.copyto(self.hv, self.hv0)

    def host_run(self):
        self.xss.keyvalue_qsort(self.hk, self.hv)

    def host_check(self):
        # sorted keys, and every value (the original index) carries its key
        idx = np.random.default_rng(5).integers(0, self.n, 1 << 16)
        return bool((self.hk[1:] >= self.hk[:-1]).all()) and \
            bool((self.hk0[self.hv[idx].astype(np.int64)] == self.hk[idx]).all())

    def host_bytes(self):
        return self.n * (self.kb + self.vb), self.n * (self.kb + self.vb)

    # CPU baseline on a bounded sample
    def cpu_sample(self, m):
        rng = np.random.default_rng(1)
        return (rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, m, dtype=np.int64),
                np.arange(m, dtype=np.uint64))

    def cpu_prep(self, sample):
        return sample[0].copy(), sample[1].copy()

    def cpu_sort(self, lib, kind, work, threads):
        k, v = work
        if kind == "reference":
            rc = lib.keyvalue_qsort(7, 6, k.ctypes.data, v.ctypes.data, k.size, 0, 0)
        else:
            rc = lib.keyvalue_qsort_mt(7, 6, k.ctypes.data, v.ctypes.data, k.size, 0, 0, threads)
        assert rc == 0

    def cpu_run(self, lib, kind, sample, threads):
        self.cpu_sort(lib, kind, self.cpu_prep(sample), threads)


class QsortF32(Workload):
    name = "qsort_f32"
    kb = 4

    def describe(self):
        return {"workload": f"qsort float32 n=2^{self.n.bit_length() - 1} uniform [-1,1), "
                            "ascending, hasnan=false", "n": self.n,
                "l2": "inputs larger than L2; input restored per step"}

    def setup(self):
        t = self.torch
        g = t.Generator(device="cuda").manual_seed(0)
        self.k0 = t.rand(self.n, dtype=t.float32, device="cuda", generator=g) * 2 - 1
        self.k = t.empty_like(self.k0)
        self.wsb = self.xss.workspace_size("qsort", "float32", self.n)
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def restore(self):
        self.k.copy_(self.k0)

    def run(self):
        self.xss.gpu_qsort("float32", self.k.data_ptr(), self.n, False, False,
                           self.ws.data_ptr(), self.wsb, self.stream.cuda_stream)

    def check(self):
        k = self.k
        ok = bool((k[1:] >= k[:-1]).all())
        ok &= bool((self.torch.sort(self.k0).values == k).all())
        return ok

    def passes(self):
        return 4

    def bytes_per_pass(self):
        return 2 * self.n * self.kb

    def bytes_model(self):
        return self.n * self.kb * (1 + 2 * self.passes())

    def host_setup(self):
        self.hk0 = self.k0.cpu().numpy()
        self.hk = self.pinned(self.n * 4, np.float32)

    def host_restore(self):
        np.copyto(self.hk, self.hk0)

    def host_run(self):
        self.xss.qsort(self.hk)

    def host_check(self):
        return bool((self.hk[1:] >= self.hk[:-1]).all())

    def host_bytes(self):
        return self.n * 4, self.n * 4

    def cpu_sample(self, m):
        return (np.random.default_rng(0).random(m, dtype=np.float32) * 2 - 1,)

    def cpu_prep(self, sample):
        return (sample[0].copy(),)

    def cpu_sort(self, lib, kind, work, threads):
        k = work[0]
        if kind == "reference":
            rc = lib.qsort(5, k.ctypes.data, k.size, 0, 0)
        else:
            rc = lib.qsort_mt(5, k.ctypes.data, k.size, 0, 0, threads)
        assert rc == 0

    def cpu_run(self, lib, kind, sample, threads):
        self.cpu_sort(lib, kind, self.cpu_prep(sample), threads)


class SegmentedSort(Workload):
    """Many independent segments sorted in one batch (plan + CUDA graph replay).

    200,000 segments with sizes log-uniform in [1, 2^18] (seed 3); int32 keys
    uniform over the full range, uint32 values = index within the segment.
    The literal distribution totals ~4.2e9 keys; --n rescales the sizes to a
    given total (e.g. 2^27)."""

    name = "segmented_sort"
    kdt, kid, kb, vb = "int32", 4, 4, 4

    def __init__(self, torch, xss, n, stream):
        super().__init__(torch, xss, n, stream)
        rng = np.random.default_rng(3)
        sizes = np.floor(2.0 ** rng.uniform(0.0, 18.0, 200_000)).astype(np.int64)
        if n and n != SEG_LITERAL:
            sizes = np.maximum(1, np.round(sizes * (n / sizes.sum()))).astype(np.int64)
        self.sizes = sizes
        self.off = np.zeros(sizes.size + 1, np.uint64)
        self.off[1:] = np.cumsum(sizes).astype(np.uint64)
        self.n = int(self.off[-1])

    def describe(self):
        keys = "int32 keys uniform full range" if self.kdt == "int32" else "float32 keys N(0,1)"
        return {"workload": f"segmented keyvalue sort, {self.sizes.size} segments, sizes "
                            f"log-uniform [1, 2^18] (seed 3), {keys} -> uint32 local index",
                "n": self.n, "segments": int(self.sizes.size),
                "l2": "inputs far larger than L2; input restored per step"}

    def setup(self):
        t, n = self.torch, self.n
        g = t.Generator(device="cuda").manual_seed(3)
        if self.kdt == "int32":
            self.k0 = t.randint(0, 256, (n * 4,), dtype=t.uint8, device="cuda",
                                generator=g).view(t.int32)
        else:
            self.k0 = t.randn(n, dtype=t.float32, device="cuda", generator=g)
        self.doff = t.from_numpy(self.off.view(np.int64).copy()).cuda()
        self.v0 = t.empty(n, dtype=t.int32, device="cuda")
        chunk = 1 << 27
        for b in range(0, n, chunk):
            idx = t.arange(b, min(n, b + chunk), dtype=t.int64, device="cuda")
            seg = t.searchsorted(self.doff, idx, right=True) - 1
            self.v0[b:b + idx.numel()] = (idx - self.doff[seg]).to(t.int32)
            del idx, seg
        self.k = t.empty_like(self.k0)
        self.v = t.empty_like(self.v0)
        self.plan = self.xss.SegPlan(self.kdt, "uint32", self.off)
        self.wsb = self.plan.workspace_size
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def restore(self):
        self.k.copy_(self.k0)
        self.v.copy_(self.v0)

    def run(self):
        self.plan.run(self.k.data_ptr(), self.v.data_ptr(), self.doff.data_ptr(),
                      self.ws.data_ptr(), self.wsb, self.stream.cuda_stream, use_graph=True)

    def run_nograph(self):
        self.plan.run(self.k.data_ptr(), self.v.data_ptr(), self.doff.data_ptr(),
                      self.ws.data_ptr(), self.wsb, self.stream.cuda_stream, use_graph=False)

    def run_percall(self):
        self.xss.gpu_segmented_sort_percall(self.kdt, "uint32", self.k.data_ptr(),
                                            self.v.data_ptr(), self.off,
                                            stream=self.stream.cuda_stream)

    def percall_leg(self, segments):
        """The same batch by one single-array call per segment, over the first
        `segments` segments (0: all).  Segment sizes are drawn i.i.d., so a
        contiguous block is a uniform sample; its time is scaled by the segment
        count.  The sampled segments' outputs must equal the batched outputs
        (this runs after check(), on the batched result of the last step)."""
        t = self.torch
        total = int(self.sizes.size)
        S = total if not segments else min(int(segments), total)
        e = int(self.off[S])
        ref_k, ref_v = self.k[:e].clone(), self.v[:e].clone()
        times = []
        for _ in range(2):           # the first run is the warm-up
            with t.cuda.stream(self.stream):
                self.k[:e].copy_(self.k0[:e])
                self.v[:e].copy_(self.v0[:e])
            e0, e1 = t.cuda.Event(enable_timing=True), t.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            self.xss.gpu_segmented_sort_percall(self.kdt, "uint32", self.k.data_ptr(),
                                                self.v.data_ptr(), self.off[:S + 1],
                                                stream=self.stream.cuda_stream)
            e1.record(self.stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        self.xss.stream_status(self.stream.cuda_stream)
        same = bool((self.k[:e] == ref_k).all()) and bool((self.v[:e] == ref_v).all())
        del ref_k, ref_v
        return {"ms_sampled": times[-1], "segments_sampled": S, "segments": total,
                "keys_sampled": e, "ms_scaled": times[-1] * total / S,
                "sample": "contiguous block of the i.i.d. segments, time scaled by segment count"
                          if S < total else "every segment",
                "identical_outputs": same}

    def check(self, samples=300):
        rng = np.random.default_rng(11)
        picks = set(rng.integers(0, self.sizes.size, samples).tolist())
        picks.update(np.argsort(self.sizes)[-3:].tolist())
        for s in picks:
            b, e = int(self.off[s]), int(self.off[s + 1])
            k = self.k[b:e].cpu().numpy()
            v = self.v[b:e].cpu().numpy().view(np.uint32)
            k0 = self.k0[b:e].cpu().numpy()
            if not (np.all(k[1:] >= k[:-1]) and np.array_equal(np.sort(v), np.arange(e - b))
                    and np.array_equal(k0[v.astype(np.int64)], k)):
                return False
        return True

    def passes(self):
        return 4

    def bytes_per_pass(self):           # over the keys in segments of the radix class
        big = self.sizes[self.sizes > 4096].sum()
        return 2 * int(big) * (self.kb + self.vb)

    def bytes_model(self):
        return self.n * (self.kb + 2 * self.passes() * (self.kb + self.vb))

    def cpu_sample(self, m):
        return None

    def cpu_run(self, lib, kind, sample, threads):
        """The reference's way: one keyvalue_qsort call per segment, on the
        first segments holding about m keys."""
        m = self._cpu_m
        stop = int(np.searchsorted(self.off, m))
        rng = np.random.default_rng(3)
        if self.kdt == "int32":
            k = rng.integers(-2**31, 2**31 - 1, int(self.off[stop]), dtype=np.int32)
        else:
            k = rng.standard_normal(int(self.off[stop])).astype(np.float32)
        v = np.zeros(k.size, np.uint32)
        for s in range(stop):
            b, e = int(self.off[s]), int(self.off[s + 1])
            v[b:e] = np.arange(e - b, dtype=np.uint32)
        for s in range(stop):
            b, e = int(self.off[s]), int(self.off[s + 1])
            if e - b <= 1:
                continue
            if kind == "reference" or e - b <= 10000:
                rc = lib.keyvalue_qsort(self.kid, 3, k[b:].ctypes.data, v[b:].ctypes.data, e - b,
                                        0, 0)
            else:   # the reference's key-value sort goes task-parallel above 1e4 keys
                rc = lib.keyvalue_qsort_mt(self.kid, 3, k[b:].ctypes.data, v[b:].ctypes.data,
                                           e - b, 0, 0, threads)
            assert rc == 0
        return int(self.off[stop])


class QsortF32Small(QsortF32):
    """qsort of 2^20 float32 keys (4 MiB, fits in L2): L2 is flushed between steps."""

    name = "qsort_f32_2e20"
    flush_l2 = True

    def describe(self):
        d = super().describe()
        d["l2"] = "input fits in L2: a 256 MiB buffer is written between steps (untimed)"
        return d


class ArgsortWorkload(Workload):
    """argsort at 2^28: int64 uniform full range ascending, or float64 ~ N(0,1)
    with 1% quiet NaN and 0.5% +-0.0, hasnan, descending."""

    name = "argsort"
    kdt = "int64"
    kb, ib = 8, 8
    desc = False

    def describe(self):
        return {"workload": f"argsort {self.kdt} n=2^{self.n.bit_length() - 1}"
                            + (" N(0,1) 1% NaN 0.5% +-0, hasnan, descending" if self.desc
                               else " uniform full range, ascending"),
                "n": self.n, "l2": "inputs larger than L2"}

    def setup(self):
        t, n = self.torch, self.n
        g = t.Generator(device="cuda").manual_seed(1)
        if self.kdt == "float64":
            x = t.randn(n, dtype=t.float64, device="cuda", generator=g)
            u = t.rand(n, dtype=t.float64, device="cuda", generator=g)
            x[u < 0.01] = float("nan")
            x[(u >= 0.01) & (u < 0.0125)] = 0.0
            x[(u >= 0.0125) & (u < 0.015)] = -0.0
            self.k0 = x
        else:
            self.k0 = t.randint(0, 256, (n * 8,), dtype=t.uint8, device="cuda",
                                generator=g).view(t.int64)
        self.arg = t.empty(n, dtype=t.int64, device="cuda")
        self.wsb = self.xss.workspace_size("argsort", self.kdt, n)
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def restore(self):
        pass                         # argsort leaves its input untouched

    def run(self):
        self.xss.gpu_argsort(self.kdt, self.k0.data_ptr(), self.arg.data_ptr(), self.n,
                             self.desc, self.desc, self.ws.data_ptr(), self.wsb,
                             self.stream.cuda_stream)

    def check(self):
        t = self.torch
        s = self.k0[self.arg]
        seen = t.zeros(self.n, dtype=t.int32, device="cuda")
        seen.index_add_(0, self.arg, t.ones(self.n, dtype=t.int32, device="cuda"))
        if self.desc:
            nan = t.isnan(s)
            c = int(nan.sum())
            r = s[c:]
            return bool(nan[:c].all()) and bool((r[1:] <= r[:-1]).all()) and bool((seen == 1).all())
        return bool((s[1:] >= s[:-1]).all()) and bool((seen == 1).all())

    def passes(self):
        return self.kb

    def bytes_per_pass(self):        # key + index read and written (index modelled 8 B)
        return 2 * self.n * (self.kb + self.ib)

    def bytes_model(self):           # n(kb + 2P(kb+ib)) - n(ib+kb)
        return self.n * (self.kb + 2 * self.passes() * (self.kb + self.ib)) - \
            self.n * (self.ib + self.kb)

    def host_setup(self):
        self.hk = self.pinned(self.n * 8, np.dtype(self.kdt))
        self.hk[:] = self.k0.cpu().numpy()
        # the indices go to the caller's pinned array (the reference's
        # argsort(T*, size_t* arg, ...) form)
        self.harg = self.pinned(self.n * 8, np.uint64)

    def host_restore(self):
        pass

    def host_run(self):
        self.xss.argsort(self.hk, self.desc, self.desc, out=self.harg)

    def host_check(self):
        # the gathered keys are in order (NaN-free sample positions)
        g = self.hk[self.harg[: 1 << 20].astype(np.int64)]
        g = g[~np.isnan(g)] if g.dtype.kind == "f" else g
        return bool((g[1:] <= g[:-1]).all()) if self.desc else bool((g[1:] >= g[:-1]).all())

    def host_bytes(self):
        return self.n * self.kb, self.n * 8

    def cpu_sample(self, m):
        rng = np.random.default_rng(1)
        if self.kdt == "float64":
            x = rng.standard_normal(m)
            u = rng.random(m)
            x[u < 0.01] = np.nan
            x[(u >= 0.01) & (u < 0.0125)] = 0.0
            x[(u >= 0.0125) & (u < 0.015)] = -0.0
            return (x,)
        return (rng.integers(np.iinfo(np.int64).min, np.iinfo(np.int64).max, m,
                             dtype=np.int64),)

    def cpu_run(self, lib, kind, sample, threads):
        x = sample[0]
        arg = np.empty(x.size, np.uint64)
        dt = 8 if self.kdt == "float64" else 7
        if kind == "reference":
            rc = lib.argsort(dt, x.ctypes.data, arg.ctypes.data, x.size, int(self.desc),
                             int(self.desc))
        else:
            rc = lib.argsort_mt(dt, x.ctypes.data, arg.ctypes.data, x.size, int(self.desc),
                                int(self.desc), threads)
        assert rc == 0


class ArgsortF64(ArgsortWorkload):
    name = "argsort_f64"
    kdt = "float64"
    desc = True


class SelectWorkload(Workload):
    """qselect / partial_qsort of 2^27 float32 keys ~ N(0,1) (seed 2) at k."""

    name = "qselect_f32"
    dominant = None
    partial = False
    kb = 4
    default_k = 1 << 26

    def describe(self):
        return {"workload": f"{'partial_qsort' if self.partial else 'qselect'} float32 "
                            f"n=2^{self.n.bit_length() - 1} N(0,1) k={self.k}",
                "n": self.n, "k": self.k, "l2": "inputs larger than L2; restored per step"}

    def setup(self):
        t = self.torch
        g = t.Generator(device="cuda").manual_seed(2)
        self.k0 = t.randn(self.n, device="cuda", generator=g)
        self.x = t.empty_like(self.k0)
        op = "partial_qsort" if self.partial else "qselect"
        self.wsb = self.xss.workspace_size(op, "float32", self.n, self.k)
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def restore(self):
        self.x.copy_(self.k0)

    def run(self):
        f = self.xss.gpu_partial_qsort if self.partial else self.xss.gpu_qselect
        f("float32", self.x.data_ptr(), self.k, self.n, False, False, self.ws.data_ptr(),
          self.wsb, self.stream.cuda_stream)

    def check(self):
        t = self.torch
        kk = self.k - 1 if self.partial else self.k
        kth = t.kthvalue(self.k0, kk + 1).values
        ok = float(self.x[kk]) == float(kth)
        ok &= bool((self.x[kk + 1:] >= self.x[kk]).all())
        if self.partial:
            ok &= bool(t.equal(self.x[:self.k], t.sort(self.k0).values[:self.k]))
        return ok

    def passes(self):
        return 1

    def bytes_per_pass(self):
        return None

    def bytes_model(self):           # histogram + one partition R+W (+ sort of the top k)
        m = 3 * self.n * self.kb
        if self.partial:
            m += self.k * self.kb * (1 + 2 * self.kb)
        return m

    def host_setup(self):
        self.hk0 = self.k0.cpu().numpy()
        self.hk = self.pinned(self.n * 4, np.float32)

    def host_restore(self):
        np.copyto(self.hk, self.hk0)

    def host_run(self):
        (self.xss.partial_qsort if self.partial else self.xss.qselect)(self.hk, self.k)

    def host_bytes(self):
        return self.n * 4, self.n * 4

    def cpu_sample(self, m):
        return (np.random.default_rng(2).standard_normal(m).astype(np.float32),)

    def cpu_run(self, lib, kind, sample, threads):
        x = sample[0].copy()
        kk = min(self.k, x.size - 1) * x.size // self.n if self.k > 1000 else min(self.k, x.size - 1)
        f = lib.partial_qsort if self.partial else lib.qselect
        assert f(5, x.ctypes.data, max(kk, 1) if self.partial else kk, x.size, 0, 0) == 0


class PartialWorkload(SelectWorkload):
    name = "partial_f32"
    partial = True



def zipf16_codes(rng, dtype):
    """4096 distinct 16-bit patterns; finite values other than -0.0 for float16."""
    if dtype == "uint16":
        return rng.choice(65536, 4096, replace=False).astype(np.uint16)
    pool = np.arange(65536, dtype=np.uint16)
    finite = pool[((pool & 0x7C00) != 0x7C00) & (pool != 0x8000)]
    return rng.choice(finite, 4096, replace=False).astype(np.uint16)


ZIPF_P = 1.0 / np.arange(1, 4097) ** 1.1
ZIPF_P /= ZIPF_P.sum()


class SelectZipf16(SelectWorkload):
    """qselect of 2^28 16-bit keys drawn Zipf(s=1.1) over 4096 distinct values
    (heavy duplicates), k = 2^20 (seed 2)."""

    name = "qselect_u16_zipf"
    kdt, kid, kb = "uint16", 0, 2
    default_k = 1 << 20

    def describe(self):
        return {"workload": f"qselect {self.kdt} n=2^{self.n.bit_length() - 1} Zipf(s=1.1) "
                            f"over 4096 distinct values k={self.k}",
                "n": self.n, "k": self.k, "l2": "inputs larger than L2; restored per step"}

    def setup(self):
        t = self.torch
        table = t.tensor(zipf16_codes(np.random.default_rng(2), self.kdt).view(np.int16),
                         device="cuda")
        cdf = t.tensor(np.cumsum(ZIPF_P), device="cuda")
        g = t.Generator(device="cuda").manual_seed(2)
        self.k0 = t.empty(self.n, dtype=t.int16, device="cuda")
        chunk = 1 << 26
        for b in range(0, self.n, chunk):
            m = min(chunk, self.n - b)
            r = t.searchsorted(cdf, t.rand(m, dtype=t.float64, device="cuda", generator=g))
            self.k0[b:b + m] = table[r.clamp(max=4095)]
            del r
        self.x = t.empty_like(self.k0)
        self.wsb = self.xss.workspace_size("qselect", self.kdt, self.n, self.k)
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def run(self):
        self.xss.gpu_qselect(self.kdt, self.x.data_ptr(), self.k, self.n, False, False,
                             self.ws.data_ptr(), self.wsb, self.stream.cuda_stream)

    def _order_key(self, a):
        t = self.torch
        if self.kdt == "uint16":
            return a.to(t.int32) & 0xFFFF
        return a.view(t.float16).to(t.float32)

    def check(self):
        t = self.torch
        kx, ky = self._order_key(self.k0), self._order_key(self.x)
        kth = t.kthvalue(kx, self.k + 1).values
        ok = float(ky[self.k]) == float(kth)
        ok &= bool((ky[:self.k] <= ky[self.k]).all()) and bool((ky[self.k + 1:] >= ky[self.k]).all())
        ok &= bool(t.equal(t.sort(ky).values, t.sort(kx).values))
        return ok

    def host_setup(self):
        hd = np.uint16 if self.kdt == "uint16" else np.float16
        self.hk0 = self.k0.cpu().numpy().view(hd)
        self.hk = self.pinned(self.n * 2, hd)

    def host_bytes(self):
        return self.n * 2, self.n * 2

    def cpu_sample(self, m):
        rng = np.random.default_rng(2)
        table = zipf16_codes(rng, self.kdt)
        return (table[rng.choice(4096, m, p=ZIPF_P)],)

    def cpu_run(self, lib, kind, sample, threads):
        x = sample[0].copy()
        kk = max(1, self.k * x.size // self.n)
        assert lib.qselect(self.kid, x.ctypes.data, kk, x.size, 0, 0) == 0


class SelectZipfF16(SelectZipf16):
    name = "qselect_f16_zipf"
    kdt, kid = "float16", 2


class KeyValueSelectWorkload(SelectWorkload):
    """keyvalue_select of 2^27 float32 keys ~ N(0,1) (seed 2) carrying uint32
    values = original index, at k."""

    name = "kv_select_f32"
    op = "keyvalue_select"
    kdt, kid, vdt, kb, vb = "float32", 5, "uint32", 4, 4
    default_k = 1 << 26

    def describe(self):
        dist = "N(0,1)" if self.kdt == "float32" else "uniform full range"
        return {"workload": f"{self.op} {self.kdt}->{self.vdt} n=2^{self.n.bit_length() - 1} "
                            f"{dist}, values=index, k={self.k}",
                "n": self.n, "k": self.k, "l2": "inputs larger than L2; restored per step"}

    def make_keys(self, g):
        return self.torch.randn(self.n, device="cuda", generator=g)

    def setup(self):
        t = self.torch
        g = t.Generator(device="cuda").manual_seed(2)
        self.k0 = self.make_keys(g)
        self.v0 = t.arange(self.n, dtype=t.int32, device="cuda")
        self.x = t.empty_like(self.k0)
        self.v = t.empty_like(self.v0)
        self.wsb = self.xss.workspace_size(self.op, self.kdt, self.n, self.k, val_dtype=self.vdt)
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def restore(self):
        self.x.copy_(self.k0)
        self.v.copy_(self.v0)

    def run(self):
        f = (self.xss.gpu_keyvalue_partial_sort if self.op == "keyvalue_partial_sort"
             else self.xss.gpu_keyvalue_select)
        f(self.kdt, self.vdt, self.x.data_ptr(), self.v.data_ptr(), self.k, self.n, False, False,
          self.ws.data_ptr(), self.wsb, self.stream.cuda_stream)

    def check(self):
        t = self.torch
        vi = self.v.to(t.int64)
        ok = bool(t.equal(self.k0[vi], self.x))
        cnt = t.zeros(self.n, dtype=t.int32, device="cuda")
        cnt.index_add_(0, vi, t.ones(self.n, dtype=t.int32, device="cuda"))
        ok &= bool((cnt == 1).all())
        kk = self.k - 1 if self.op == "keyvalue_partial_sort" else self.k
        kth = t.kthvalue(self.k0, kk + 1).values
        ok &= float(self.x[kk]) == float(kth)
        ok &= bool((self.x[:kk] <= self.x[kk]).all()) and bool((self.x[kk + 1:] >= self.x[kk]).all())
        if self.op == "keyvalue_partial_sort":
            ok &= bool(t.equal(self.x[:self.k], t.sort(self.k0).values[:self.k]))
        return ok

    def bytes_model(self):    # histogram + one partition of the pairs R+W (+ sort of the top k)
        m = self.n * self.kb + 2 * self.n * (self.kb + self.vb)
        if self.op == "keyvalue_partial_sort":
            m += self.k * (self.kb + 2 * self.kb * (self.kb + self.vb))
        return m

    def host_setup(self):
        self.hk0 = self.k0.cpu().numpy()
        self.hv0 = self.v0.cpu().numpy().view(np.uint32)
        self.hk = self.pinned(self.n * self.kb, self.hk0.dtype)
        self.hv = self.pinned(self.n * self.vb, np.uint32)

    def host_restore(self):
        np.copyto(self.hk, self.hk0)
        np.copyto(self.hv, self.hv0)

    def host_run(self):
        f = (self.xss.keyvalue_partial_sort if self.op == "keyvalue_partial_sort"
             else self.xss.keyvalue_select)
        f(self.hk, self.hv, self.k)

    def host_bytes(self):
        return self.n * (self.kb + self.vb), self.n * (self.kb + self.vb)

    def cpu_sample(self, m):
        rng = np.random.default_rng(2)
        if self.kdt == "float32":
            k = rng.standard_normal(m).astype(np.float32)
        else:
            k = rng.integers(-2**31, 2**31 - 1, m, dtype=np.int32)
        return (k, np.arange(m, dtype=np.uint32))

    def cpu_run(self, lib, kind, sample, threads):
        k, v = sample[0].copy(), sample[1].copy()
        if self.op == "keyvalue_partial_sort":
            rc = lib.keyvalue_partial_sort(self.kid, 3, k.ctypes.data, v.ctypes.data, self.k,
                                           k.size, 0, 0)
        else:
            kk = max(1, self.k * k.size // self.n)
            rc = lib.keyvalue_select(self.kid, 3, k.ctypes.data, v.ctypes.data, kk, k.size, 0, 0)
        assert rc == 0


class KeyValuePartialI32(KeyValueSelectWorkload):
    """keyvalue_partial_sort of 2^27 int32 keys (uniform full range, seed 2)
    carrying uint32 values = original index, k = 4096."""

    name = "kv_partial_i32"
    op = "keyvalue_partial_sort"
    kdt, kid = "int32", 4
    default_k = 4096

    def make_keys(self, g):
        t = self.torch
        return t.randint(-2**31, 2**31 - 1, (self.n,), dtype=t.int32, device="cuda", generator=g)


class ArgselectF32(SelectWorkload):
    """argselect of 2^27 float32 keys ~ N(0,1) (seed 2) at k: 64-bit indices,
    the input left as it is."""

    name = "argselect_f32"
    default_k = 1 << 26

    def describe(self):
        return {"workload": f"argselect float32 n=2^{self.n.bit_length() - 1} N(0,1) k={self.k}",
                "n": self.n, "k": self.k, "l2": "inputs larger than L2"}

    def setup(self):
        t = self.torch
        g = t.Generator(device="cuda").manual_seed(2)
        self.k0 = t.randn(self.n, device="cuda", generator=g)
        self.arg = t.empty(self.n, dtype=t.int64, device="cuda")
        self.wsb = self.xss.workspace_size("argselect", "float32", self.n, self.k)
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def restore(self):
        self.arg.fill_(-1)

    def run(self):
        self.xss.gpu_argselect("float32", self.k0.data_ptr(), self.arg.data_ptr(), self.k,
                               self.n, False, self.ws.data_ptr(), self.wsb,
                               self.stream.cuda_stream)

    def check(self):
        t = self.torch
        a = self.arg
        ok = bool(((a >= 0) & (a < self.n)).all())
        if not ok:
            return False
        cnt = t.zeros(self.n, dtype=t.int32, device="cuda")
        cnt.index_add_(0, a, t.ones(self.n, dtype=t.int32, device="cuda"))
        ok &= bool((cnt == 1).all())
        x = self.k0[a]
        kth = t.kthvalue(self.k0, self.k + 1).values
        ok &= float(x[self.k]) == float(kth)
        ok &= bool((x[:self.k] <= kth).all()) and bool((x[self.k + 1:] >= kth).all())
        return ok

    def bytes_model(self):    # histogram + one partition of (key, 64-bit index) R+W
        return self.n * 4 + 2 * self.n * (4 + 8)

    def host_setup(self):
        self.hk = self.pinned(self.n * 4, np.float32)
        np.copyto(self.hk, self.k0.cpu().numpy())
        self.harg = self.pinned(self.n * 8, np.uint64)   # the caller's index array

    def host_restore(self):
        pass

    def host_run(self):
        self.xss.argselect(self.hk, self.k, out=self.harg)

    def host_bytes(self):
        return self.n * 4, self.n * 8

    def cpu_run(self, lib, kind, sample, threads):
        x = sample[0]
        arg = np.empty(x.size, np.uint64)
        kk = max(1, self.k * x.size // self.n)
        assert lib.argselect(5, x.ctypes.data, arg.ctypes.data, kk, x.size, 0) == 0


class ObjectRecords(Workload):
    """Device object sort: 2^26 records of 24 bytes {int32 x, int32 y, float32
    distance, 4 pad bytes, uint64 metric}, y = original position, ordered by the
    float32 member `distance` ~ N(0,1) (seed 5) through xss_gpu_object_qsort."""

    name = "object_records"
    kb, rec, key_off = 4, 24, 8
    dominant = None

    def describe(self):
        return {"workload": f"object_qsort of n=2^{self.n.bit_length() - 1} device records of 24 B "
                            "{int32 x, int32 y, float32 distance, uint64 metric} by distance "
                            "~ N(0,1)", "n": self.n,
                "l2": "inputs larger than L2; restored per step"}

    def setup(self):
        t, n = self.torch, self.n
        g = t.Generator(device="cuda").manual_seed(5)
        w = t.zeros((n, 6), dtype=t.int32, device="cuda")
        w[:, 0] = t.randint(-1000, 1000, (n,), dtype=t.int32, device="cuda", generator=g)
        w[:, 1] = t.arange(n, dtype=t.int32, device="cuda")
        w[:, 2] = t.randn(n, device="cuda", generator=g).view(t.int32)
        w[:, 4:6] = t.randint(0, 2**31 - 1, (n, 2), dtype=t.int32, device="cuda", generator=g)
        self.r0 = w.view(-1)
        self.r = t.empty_like(self.r0)
        self.wsb = self.xss.object_workspace_size(n, self.rec, "float32")
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def restore(self):
        self.r.copy_(self.r0)

    def run(self):
        self.xss.gpu_object_qsort(self.r.data_ptr(), self.n, self.rec, self.key_off, "float32",
                                  False, False, self.ws.data_ptr(), self.wsb,
                                  self.stream.cuda_stream)

    def check(self):
        t = self.torch
        w0, w = self.r0.view(self.n, 6), self.r.view(self.n, 6)
        d = w[:, 2].contiguous().view(t.float32)
        ok = bool((d[1:] >= d[:-1]).all())
        src = w[:, 1].to(t.int64)
        ok &= bool(((src >= 0) & (src < self.n)).all())
        if not ok:
            return False
        cnt = t.zeros(self.n, dtype=t.int32, device="cuda")
        cnt.index_add_(0, src, t.ones(self.n, dtype=t.int32, device="cuda"))
        ok &= bool((cnt == 1).all())
        ok &= bool(t.equal(w0[src], w))
        return ok

    def passes(self):
        return 4

    def bytes_per_pass(self):
        return 2 * self.n * (self.kb + 4)

    def bytes_model(self):
        # key read (every sector of the records holds a key) + (key, position)
        # written, their key-value sort, the record gather R+W and the copy back
        n, r = self.n, self.rec
        return n * r + n * (self.kb + 4) + n * (self.kb + 2 * 4 * (self.kb + 4)) + 4 * n * r

    def cpu_sample(self, m):
        rng = np.random.default_rng(5)
        w = np.zeros((m, 6), np.int32)
        w[:, 0] = rng.integers(-1000, 1000, m)
        w[:, 1] = np.arange(m)
        w[:, 2] = rng.standard_normal(m).astype(np.float32).view(np.int32)
        return (w,)

    def cpu_run(self, lib, kind, sample, threads):
        """The reference's object_qsort: keys read out of the objects, a key-value
        sort of (key, position), then the objects permuted."""
        w = sample[0].copy()
        keys = w[:, 2].copy().view(np.float32)
        pos = np.arange(w.shape[0], dtype=np.uint32)
        if kind == "reference":
            rc = lib.keyvalue_qsort(5, 3, keys.ctypes.data, pos.ctypes.data, keys.size, 0, 0)
        else:
            rc = lib.keyvalue_qsort_mt(5, 3, keys.ctypes.data, pos.ctypes.data, keys.size, 0, 0,
                                       threads)
        assert rc == 0
        w[:] = w[pos]


class ObjectPoint3D(ObjectRecords):
    """object_qsort of Point3D<double> {x, y, z} records (24 B) by the member x,
    uniform [0, 1) doubles (seed 5): the shape of the reference's published
    object-sort benchmark (misc/bench-simdobjsort.txt:16,23: n = 1,048,576 in
    51.58 ms, n = 1e8 in 15.53 s on an unspecified AVX-512 processor).  Device
    form (xss_gpu_object_qsort); e2e adds the copy of the records in and out."""

    name = "object_point3d"
    kb, rec, key_off = 8, 24, 0
    flush_l2 = True
    published = {1 << 20: (1 << 20) / 51.58e-3 / 1e9, 100_000_000: 1e8 / 15.53 / 1e9}
    published_source = "misc/bench-simdobjsort.txt:16,23 (object_qsort Point3D<double> by x)"

    def describe(self):
        return {"workload": f"object_qsort of n={self.n} Point3D<double> records (24 B) by x, "
                            "uniform [0,1)", "n": self.n,
                "l2": "inputs restored per step; a 256 MiB buffer is written between steps "
                      "(untimed), as 2^20 records fit in L2"}

    def setup(self):
        t, n = self.torch, self.n
        g = t.Generator(device="cuda").manual_seed(5)
        self.p0 = t.rand((n, 3), dtype=t.float64, device="cuda", generator=g)
        self.r0 = self.p0.view(-1)
        self.r = t.empty_like(self.r0)
        self.wsb = self.xss.object_workspace_size(n, self.rec, "float64")
        self.ws = t.empty(max(self.wsb, 1), dtype=t.uint8, device="cuda")

    def run(self):
        self.xss.gpu_object_qsort(self.r.data_ptr(), self.n, self.rec, self.key_off, "float64",
                                  False, False, self.ws.data_ptr(), self.wsb,
                                  self.stream.cuda_stream)

    def check(self):
        t = self.torch
        w = self.r.view(self.n, 3)
        order = t.sort(self.p0[:, 0], stable=True).indices
        return bool(t.equal(self.p0[order], w))

    def bytes_per_pass(self):
        return 2 * self.n * (self.kb + 4)

    def bytes_model(self):
        n, r = self.n, self.rec
        return n * r + n * (self.kb + 4) + n * (self.kb + 2 * 8 * (self.kb + 4)) + 4 * n * r

    def host_setup(self):
        self.hr0 = self.p0.cpu().numpy().reshape(-1)
        self.hr = self.pinned(self.n * self.rec, np.float64)
        self.hr_t = self._pinned[-1]          # the pinned tensor behind self.hr

    def host_restore(self):
        np.copyto(self.hr, self.hr0)

    def host_run(self):
        t = self.torch
        dev = self.r.view(t.uint8)
        with t.cuda.stream(self.stream):
            dev.copy_(self.hr_t, non_blocking=True)
            self.run()
            self.hr_t.copy_(dev, non_blocking=True)
        self.stream.synchronize()

    def host_bytes(self):
        return self.n * self.rec, self.n * self.rec

    def cpu_sample(self, m):
        return (np.random.default_rng(5).random((m, 3)),)

    def cpu_run(self, lib, kind, sample, threads):
        w = sample[0].copy()
        keys = w[:, 0].copy()
        pos = np.arange(w.shape[0], dtype=np.uint32)
        if kind == "reference":
            rc = lib.keyvalue_qsort(8, 3, keys.ctypes.data, pos.ctypes.data, keys.size, 0, 0)
        else:
            rc = lib.keyvalue_qsort_mt(8, 3, keys.ctypes.data, pos.ctypes.data, keys.size, 0, 0,
                                       threads)
        assert rc == 0
        w[:] = w[pos]


class SegmentedF32(SegmentedSort):
    """The float32 variant of the segmented batch: keys ~ N(0,1)."""

    name = "segmented_f32"
    kdt, kid = "float32", 5


class SegmentedTopk(SegmentedSort):
    """Batched top-k over the config-4 segments (int32 keys -> uint32 local
    index): every segment's k smallest keys, in order, at its front
    (xss_gpu_segmented_topk).  Segments up to 4096 keys are sorted whole on
    chip; longer ones are streamed once by one CTA each (k <= 2048)."""

    name = "segmented_topk"
    default_k = 1000
    dominant = None
    has_percall = False
    roofline_name = "segmented top-k (all kernels of one call)"

    def describe(self):
        d = super().describe()
        d["workload"] = d["workload"].replace("segmented keyvalue sort",
                                              f"segmented keyvalue top-k, k={self.k},")
        d["k"] = self.k
        return d

    def run(self):
        self.xss.gpu_segmented_topk(self.kdt, "uint32", self.kk.data_ptr(), self.v.data_ptr(),
                                    self.doff.data_ptr(), self.off, self.sizes.size, self.k,
                                    False, False, self.ws.data_ptr(), self.wsb,
                                    self.stream.cuda_stream)

    def setup(self):
        topk = self.k
        super().setup()                  # names the key buffer self.k
        self.kk, self.k = self.k, topk   # key buffer; the workload's k

    def restore(self):
        self.kk.copy_(self.k0)
        self.v.copy_(self.v0)

    def check(self, samples=300):
        rng = np.random.default_rng(11)
        picks = set(rng.integers(0, self.sizes.size, samples).tolist())
        picks.update(np.argsort(self.sizes)[-3:].tolist())
        for s in picks:
            b, e = int(self.off[s]), int(self.off[s + 1])
            m = min(self.k, e - b)
            k = self.kk[b:e].cpu().numpy()
            v = self.v[b:e].cpu().numpy().view(np.uint32)
            k0 = self.k0[b:e].cpu().numpy()
            if not (np.array_equal(k[:m], np.sort(k0)[:m])
                    and np.array_equal(np.sort(v), np.arange(e - b))
                    and np.array_equal(k0[v.astype(np.int64)], k)):
                return False
        return True

    def cpu_run(self, lib, kind, sample, threads):
        """The reference's way: one keyvalue_partial_sort(k) call per segment,
        on the first segments holding about m keys (single-threaded: the
        reference's partial sorts are not task-parallel)."""
        m = self._cpu_m
        stop = int(np.searchsorted(self.off, m))
        rng = np.random.default_rng(3)
        k = rng.integers(-2**31, 2**31 - 1, int(self.off[stop]), dtype=np.int32)
        v = np.zeros(k.size, np.uint32)
        for s in range(stop):
            b, e = int(self.off[s]), int(self.off[s + 1])
            v[b:e] = np.arange(e - b, dtype=np.uint32)
        for s in range(stop):
            b, e = int(self.off[s]), int(self.off[s + 1])
            if e - b <= 1:
                continue
            rc = lib.keyvalue_partial_sort(self.kid, 3, k[b:].ctypes.data, v[b:].ctypes.data,
                                           min(self.k, e - b), e - b, 0, 0)
            assert rc == 0
        return int(self.off[stop])

    def passes(self):
        return 1

    def bytes_model(self):
        """One read of every key of the streamed segments; a read and a write
        of keys and values for the segments sorted whole, for each streamed
        segment's first 4096 keys and for its k results."""
        small = self.sizes[self.sizes <= 4096]
        big = self.sizes[self.sizes > 4096]
        rw = self.kb + self.vb
        return int(2 * small.sum() * rw + big.sum() * self.kb +
                   big.size * 2 * (4096 + self.k) * rw)

    def bytes_per_pass(self):
        return self.bytes_model()

SEG_LITERAL = -1
DTYPE_OF = {"keyvalue_qsort": "int64", "qsort_f32": "f32", "segmented": "int32",
            "qsort_f32_2e20": "f32", "argsort_i64": "int64", "argsort_f64": "f64",
            "segmented_topk": "int32",
            "qselect_f32": "f32", "partial_f32": "f32", "segmented_f32": "f32",
            "qselect_u16_zipf": "u16", "qselect_f16_zipf": "f16", "kv_select_f32": "f32",
            "kv_partial_i32": "int32", "argselect_f32": "f32", "object_records": "f32",
            "object_point3d": "f64"}
WORKLOADS = {"keyvalue_qsort": (KeyValueSort, 1 << 28), "qsort_f32": (QsortF32, 1 << 28),
             "segmented": (SegmentedSort, SEG_LITERAL),
             "qsort_f32_2e20": (QsortF32Small, 1 << 20),
             "argsort_i64": (ArgsortWorkload, 1 << 28), "argsort_f64": (ArgsortF64, 1 << 28),
             "qselect_f32": (SelectWorkload, 1 << 27), "partial_f32": (PartialWorkload, 1 << 27),
             "segmented_f32": (SegmentedF32, SEG_LITERAL),
             "segmented_topk": (SegmentedTopk, SEG_LITERAL),
             "qselect_u16_zipf": (SelectZipf16, 1 << 28),
             "qselect_f16_zipf": (SelectZipfF16, 1 << 28),
             "kv_select_f32": (KeyValueSelectWorkload, 1 << 27),
             "kv_partial_i32": (KeyValuePartialI32, 1 << 27),
             "argselect_f32": (ArgselectF32, 1 << 27),
             "object_records": (ObjectRecords, 1 << 26),
             "object_point3d": (ObjectPoint3D, 1 << 20)}


# ---------------------------------------------------------------------------
def cpu_baseline(wl, budget_s=12.0, sample_n=1 << 24):
    """Time the reference (where it builds here) or the oracle's port on a sample."""
    from oracle import pyoracle
    lib, kind = pyoracle.reference(), "reference"
    if lib is None:
        lib, kind = pyoracle.oracle(), "port"
    threads = pyoracle.oracle().max_threads()
    wl._cpu_m = sample_n
    sample = wl.cpu_sample(sample_n)
    times = []
    t_end = time.perf_counter() + budget_s
    done = sample_n
    while time.perf_counter() < t_end or len(times) < 2:
        t0 = time.perf_counter()
        r = wl.cpu_run(lib, kind, sample, threads)
        times.append(time.perf_counter() - t0)
        if isinstance(r, int):
            done = r
        if len(times) >= 10:
            break
    med = statistics.median(times)
    return {"value": done / med / 1e9, "unit": "Gkeys/s", "cores": threads if kind == "port"
            else min(16, os.cpu_count() or 1), "kind": kind,
            "sample": f"{wl.name} on {sample_n} keys (2^{sample_n.bit_length() - 1}), "
                      f"median of {len(times)} runs"}


# The reference's own numbers for these workloads, measured on an x86 host
# (built from its sources with g++ 13.3, AVX-512 dispatch, OpenMP on 8 threads of
# an x86 Xeon @ 2.70 GHz; single wall-clock runs).  Its SIMD code needs x86-64
# and its sources do not travel with this repository, so on other hosts the
# reference arm times the oracle's port and reports these beside it.
X86_REFERENCE_FIGURES = {
    "keyvalue_qsort": {"value": 0.1175, "unit": "Gkeys/s", "n": 1 << 28,
                       "what": "keyvalue_qsort<int64,uint64> ascending, 2^28 in 2.28 s"},
    "argsort_i64": {"value": 0.0225, "unit": "Gkeys/s", "n": 1 << 28,
                    "what": "argsort<int64> ascending, 2^28 in 11.9 s"},
    "qsort_f32": {"value": 0.492, "unit": "Gkeys/s", "n": 1 << 26,
                  "what": "qsort<float> U[-1,1), 2^26 in 136 ms"},
    "qsort_f32_2e20": {"value": 0.721, "unit": "Gkeys/s", "n": 1 << 20,
                       "what": "qsort<float> U[-1,1), 2^20 in 1.45 ms"},
    "argsort_f64": {"value": 0.0031, "unit": "Gkeys/s", "n": 1 << 24,
                    "what": "argsort<double> hasnan descending 1% NaN (scalar fallback), "
                            "2^24 in 5.39 s"},
}
X86_REFERENCE_HOST = "x86 host: 8 threads (OpenMP), Intel Xeon @ 2.70 GHz, AVX-512"


def reference_arm(args):
    """--impl reference: the reference's CPU path on the workload, timed on the
    host cores.  Where one step at the full size fits the time budget
    (--ref-budget-s for all timed steps, estimated from a timed sample) every
    timed step sorts the whole workload; otherwise a bounded sample.  Inputs
    are restored outside the timed region where the workload separates the
    copy from the sort (cpu_prep / cpu_sort)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import torch  # noqa: F401  (only for the workload class' sample helpers)
    cls, n_full = WORKLOADS[args.workload]
    wl = cls(None, None, n_full, None)
    n_full = wl.n
    if hasattr(wl, "default_k"):
        wl.k = args.k if args.k is not None else wl.default_k
    from oracle import pyoracle
    lib, kind = pyoracle.reference(), "reference"
    if lib is None:
        lib, kind = pyoracle.oracle(), "port"
    threads = pyoracle.oracle().max_threads()
    split = hasattr(wl, "cpu_sort")

    def timed(sample, m):
        wl._cpu_m = m
        if split:
            work = wl.cpu_prep(sample)
            t0 = time.perf_counter()
            r = wl.cpu_sort(lib, kind, work, threads)
            return time.perf_counter() - t0, r
        t0 = time.perf_counter()
        r = wl.cpu_run(lib, kind, sample, threads)
        return time.perf_counter() - t0, r

    m = min(args.cpu_sample, n_full)
    sample = wl.cpu_sample(m)
    t_m = 0.0
    for _ in range(max(args.warmup, 1)):     # (at least one run for the estimate)
        t_m, _ = timed(sample, m)
    if split and m < n_full and not args.ref_sample_only:
        # n log n growth from the sample to the full size
        est = t_m * (n_full / m) * (np.log2(n_full) / np.log2(m))
        if est * args.steps <= args.ref_budget_s:
            m = n_full
            sample = wl.cpu_sample(m)
    dt = 0.0
    done = 0
    for _ in range(args.steps):
        t, r = timed(sample, m)
        dt += t
        done += r if isinstance(r, int) else m
    val = done / dt / 1e9
    cores = threads if kind == "port" else min(16, os.cpu_count() or 1)
    label = ("the oracle's task-parallel port of the reference's OpenMP quicksort "
             "(the reference's SIMD paths need x86-64)" if kind == "port"
             else "the reference library built from its sources")
    line = {"impl": "reference", "metric": "Gkeys/s", "value": val, "unit": "Gkeys/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": DTYPE_OF[args.workload],
            "data": "synthetic",
            "config": {**wl.describe(), "parallelism": "replicas x1",
                       "reference_sample": ("the full workload per step" if m == n_full
                                            else f"bounded CPU sample of {m} keys per step"),
                       "same_config": m == n_full},
            "cpu_baseline": {"value": val, "unit": "Gkeys/s", "cores": cores, "kind": kind,
                             "what": label, "host": os.uname().machine,
                             "sample": f"{m} keys per step",
                             "input_restore": "outside the timed region" if split
                                              else "inside the timed region"},
            "e2e": {"value": val, "unit": "Gkeys/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    if args.workload in X86_REFERENCE_FIGURES:
        line["reference_x86_host"] = {**X86_REFERENCE_FIGURES[args.workload],
                                      "host": X86_REFERENCE_HOST,
                                      "source": "the reference built and run on an x86 host; "
                                                "not on this host"}
    print(json.dumps(line), flush=True)


def max_over_ranks(value: float, dist, device: str) -> float:
    """The slowest rank's time: every rank gets the maximum over all ranks."""
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(n_per_rank: int, ms_per_step: float, world: int) -> float:
    """Gkeys/s of N independent replicas, each sorting n_per_rank keys per step,
    timed by the slowest rank."""
    return world * n_per_rank / (ms_per_step / 1e3) / 1e9


def serving_line(args, duration=None):
    """Serving loop under Poisson load (offered 20k req/s by default).

    Mix: 45% qsort, 25% argsort, 20% qselect (k uniform in [0, n)), 10%
    keyvalue_qsort; sizes log-uniform in [2^10, 2^26]; key types uniform over
    {float32, int64, float16, float64, uint32} (32/64-bit only for key-value);
    float keys ~ N(0,1) with 0.1% NaN, hasnan = true; seed 4.  Inputs are read
    from shared pinned source arrays, results land in a pinned output ring; a
    request that finds the ring or the server queue full is shed."""
    import torch
    import pyxss as xss
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    rng = np.random.default_rng(4)
    nmax = 1 << 26
    dts = ["float32", "int64", "float16", "float64", "uint32"]
    src = {}
    for dt in dts:
        d = np.dtype(dt)
        t = torch.empty(nmax * d.itemsize, dtype=torch.uint8, pin_memory=True)
        a = t.numpy().view(d)
        if d.kind == "f":
            a[:] = rng.standard_normal(nmax).astype(d)
            a[rng.random(nmax) < 0.001] = np.nan
        else:
            a[:] = rng.integers(np.iinfo(d).min, np.iinfo(d).max, nmax, dtype=d, endpoint=True)
        src[dt] = (t, a)
    vt = torch.empty(nmax * 8, dtype=torch.uint8, pin_memory=True)
    vsrc = vt.numpy().view(np.uint64)
    vsrc[:] = np.arange(nmax, dtype=np.uint64)
    ring_bytes = args.ring_gb << 30
    ring_t = torch.empty(ring_bytes, dtype=torch.uint8, pin_memory=True)
    ring = ring_t.numpy()
    srv = xss.Server(hbm_budget_bytes=args.serve_budget_gb << 30, small_max=1 << 14,
                     max_queue=args.serve_queue, streams=args.serve_streams)
    peak, peak_src = _peaks()

    head = tail = 0          # ring bytes [tail, head) are in use, FIFO order
    inflight = []            # (ticket, ring_end, bytes_model, check)
    offered = shed_client = submitted = 0
    model_bytes_done = 0
    clocks = Clocks(int(os.environ.get("LOCAL_RANK", "0")))
    t_start = time.perf_counter()
    t_next = t_start
    duration = args.duration if duration is None else duration
    deadline = t_start + duration
    samples = []
    while True:
        now = time.perf_counter()
        # retire finished requests in FIFO order to free ring space
        while inflight:
            st = srv.poll(inflight[0][0])
            if st is None:
                break
            tk, end, mb, chk = inflight.pop(0)
            assert st == 0, st
            tail = end
            model_bytes_done += mb
            if chk is not None and len(samples) < 64:
                samples.append(chk())
        if not inflight:
            head = tail = 0
        if now >= deadline:
            break
        if now < t_next:
            time.sleep(min(t_next - now, 200e-6))
            continue
        t_next += rng.exponential(1.0 / args.rate)
        offered += 1
        u = rng.random()
        op = ("qsort" if u < 0.45 else "argsort" if u < 0.70 else "qselect" if u < 0.90
              else "keyvalue_qsort")
        dt = dts[rng.integers(0, len(dts))]
        if op == "keyvalue_qsort" and dt == "float16":
            dt = "float32"
        n = int(2.0 ** rng.uniform(10, 26))
        kb = np.dtype(dt).itemsize
        out_b = n * (8 if op == "argsort" else kb) + (n * 8 if op == "keyvalue_qsort" else 0)
        out_b = (out_b + 255) // 256 * 256
        if out_b > ring_bytes - head:
            if tail >= out_b and not inflight:
                head = tail = 0
            shed_client += 1
            continue
        o = head
        head += out_b
        a = src[dt][1]
        kw = dict(n=n, hasnan=np.dtype(dt).kind == "f")
        pout = ring[o:].ctypes.data
        if op == "argsort":
            t = srv.submit(op, dt, a.ctypes.data, None, arg_out=pout, **kw)
            mb = n * (kb + 2 * kb * (kb + 8)) - n * (8 + kb)
        elif op == "keyvalue_qsort":
            t = srv.submit(op, dt, a.ctypes.data, pout, vals_in=vsrc.ctypes.data,
                           vals_out=pout + n * kb, val_dtype="uint64", **kw)
            mb = n * (kb + 2 * kb * (kb + 8))
        elif op == "qselect":
            t = srv.submit(op, dt, a.ctypes.data, pout, k=int(rng.integers(0, n)), **kw)
            mb = 3 * n * kb
        else:
            t = srv.submit(op, dt, a.ctypes.data, pout, **kw)
            mb = n * kb * (1 + 2 * kb)
        if t is None:
            head -= out_b
            continue
        submitted += 1
        chk = None
        if op == "qsort" and n <= (1 << 16) and len(samples) < 64:
            view = ring[o:o + n * kb].view(np.dtype(dt))
            base = a[:n].copy()
            chk = (lambda v=view, b=base, d=dt: bool(np.array_equal(
                np.isnan(v) if np.dtype(d).kind == "f" else v,
                np.isnan(np.sort(b)) if np.dtype(d).kind == "f" else np.sort(b))))
        inflight.append((t, head, mb, chk))
    for tk, end, mb, chk in inflight:
        assert srv.wait(tk) == 0
        model_bytes_done += mb
    wall = time.perf_counter() - t_start
    clk = clocks.stop()
    st = srv.stats()
    srv.close()
    shed_total = shed_client + st["shed"]
    line = {
        "metric": "serving Gkeys/s with p50/p99 latency", "value": st["keys"] / wall / 1e9,
        "unit": "Gkeys/s", "n_gpus": 1, "steps": 1, "warmup": 0, "ms_per_step": wall * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "mixed",
        "data": "synthetic (seeded Poisson arrivals, seed 4)",
        "config": {"workload": "serving loop", "offered_req_per_s": args.rate,
                   "duration_s": duration, "mix": "45% qsort, 25% argsort, 20% qselect, "
                   "10% keyvalue_qsort", "sizes": "log-uniform [2^10, 2^26]",
                   "dtypes": dts, "hbm_pool_gb": args.serve_budget_gb,
                   "ring_gb": args.ring_gb, "streams": args.serve_streams,
                   "queue_limit": args.serve_queue},
        "serving": {"offered": offered, "submitted": submitted,
                    "shed": shed_total, "shed_fraction": shed_total / max(offered, 1),
                    "completed": st["completed"], "failed": st["failed"],
                    "completed_req_per_s": st["completed"] / wall,
                    "batches": st["batches"], "batched_requests": st["batched_requests"],
                    "p50_ms": st["p50_us"] / 1e3, "p99_ms": st["p99_us"] / 1e3,
                    "max_ms": st["max_us"] / 1e3,
                    "hbm_frac_model": model_bytes_done / wall / 1e9 / peak,
                    "peak_source": peak_src,
                    "checked_samples": len(samples), "checked_ok": all(samples)},
        "clocks": clk,
        "checked": bool(samples) and all(samples),
    }
    return line


def run_serving(args):
    print(json.dumps(serving_line(args)), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--workload", default="keyvalue_qsort",
                    choices=sorted(WORKLOADS) + ["serving"])
    ap.add_argument("--k", type=int, default=None,
                    help="select workloads: k (default: the workload's own)")
    ap.add_argument("--rate", type=float, default=20000.0, help="serving: offered req/s")
    ap.add_argument("--duration", type=float, default=2.0, help="serving: seconds of arrivals")
    ap.add_argument("--ring-gb", type=int, default=16, help="serving: pinned output ring")
    ap.add_argument("--serve-budget-gb", type=int, default=64, help="serving: device pool")
    ap.add_argument("--serve-streams", type=int, default=4, help="serving: request streams")
    ap.add_argument("--serve-queue", type=int, default=32, help="serving: queue limit")
    ap.add_argument("--n", type=int, default=0, help="override the array size")
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample", type=int, default=1 << 24)
    ap.add_argument("--ref-budget-s", type=float, default=150.0,
                    help="reference arm: time budget of the timed steps at the full size")
    ap.add_argument("--ref-sample-only", action="store_true",
                    help="reference arm: always time the bounded sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-percall", action="store_true",
                    help="segmented: skip the per-segment-call comparison")
    ap.add_argument("--percall-segments", type=int, default=20000,
                    help="segmented: per-call leg over the first N segments, scaled "
                         "(0: every segment)")
    ap.add_argument("--no-extras", action="store_true",
                    help="default workload: skip the f32 / segmented / serving measurements")
    ap.add_argument("--extras-serving-s", type=float, default=2.0,
                    help="seconds of arrivals of the serving measurement in the default run")
    args = ap.parse_args()
    assert args.warmup >= 3 or args.impl == "reference", "at least 3 warm-up steps"

    if args.workload == "serving" and args.impl == "ours":
        run_serving(args)
        return
    if args.impl == "reference":
        reference_arm(args)
        return

    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import pyxss as xss
    xss.lib()
    ctx = dict(torch=torch, xss=xss, dist=dist, world=world, rank=rank, local=local)
    res = measure(args, ctx, args.workload, args.n, args.steps, args.warmup,
                  do_e2e=not args.no_e2e, do_cpu=not args.no_cpu_baseline,
                  percall_segments=None if args.no_percall else args.percall_segments)
    extras = None
    if (args.workload == "keyvalue_qsort" and not args.n and not args.no_extras
            and world == 1 and rank == 0):
        extras = measure_extras(args, ctx)
    if rank == 0:
        line = res["line"]
        if extras is not None:
            line["extras"] = extras
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def measure(args, ctx, workload, n_override, steps, warmup, do_e2e=True, do_cpu=True,
            percall_segments=None):
    """One device-resident workload: W untimed warm-up steps, then K steps timed
    with CUDA events on the launching stream (input restored before each step,
    outside the events); the slowest rank's time when several ranks run.
    Returns {"line": the contract's JSON object for this workload}."""
    torch, xss, dist = ctx["torch"], ctx["xss"], ctx["dist"]
    world, rank, local = ctx["world"], ctx["rank"], ctx["local"]
    cls, n_full = WORKLOADS[workload]
    n = n_override or n_full
    stream = torch.cuda.Stream()
    wl = cls(torch, xss, n, stream)
    n = wl.n
    if hasattr(wl, "default_k"):
        wl.k = args.k if args.k is not None else wl.default_k
    flush = None
    if getattr(wl, "flush_l2", False):
        flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    with torch.cuda.stream(stream):
        wl.setup()
    torch.cuda.synchronize()

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(warmup):
        with torch.cuda.stream(stream):
            wl.restore()
            wl.run()
    xss.stream_status(stream.cuda_stream)

    xss.prof_enable(True)
    xss.prof_reset()
    launches0 = xss.prof_launches()
    clocks = Clocks(local)
    barrier()
    total_ms = 0.0
    t_wall = time.perf_counter()
    for _ in range(steps):
        with torch.cuda.stream(stream):
            wl.restore()
            if flush is not None:
                flush.zero_()        # evict the input from L2 (untimed)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        with torch.cuda.stream(stream):
            wl.run()
        e1.record(stream)
        e1.synchronize()
        total_ms += e0.elapsed_time(e1)
    barrier()
    wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    launches = xss.prof_launches() - launches0
    # event-timed device time per kernel kind (per step), the breakdown behind ms_per_step
    kernels = {}
    for kind in xss.PROF_KINDS:
        k_ms, k_n = xss.prof_read(kind)
        if k_n:
            kernels[kind] = {"ms_per_step": k_ms / steps, "launches_per_step": k_n / steps}
    dom_ms, dom_launches = xss.prof_read(wl.dominant) if wl.dominant else (0.0, 0)
    dom_steps = steps
    if dom_launches == 0 and wl.dominant and hasattr(wl, "run_nograph"):
        # kernels inside a replayed graph cannot be bracketed by events: time
        # the dominant kernel in one untimed run of the same launch sequence
        with torch.cuda.stream(stream):
            wl.restore()
        torch.cuda.synchronize()
        xss.prof_reset()
        with torch.cuda.stream(stream):
            wl.run_nograph()
        stream.synchronize()
        dom_ms, dom_launches = xss.prof_read(wl.dominant)
        dom_steps = 1
        # per-kind breakdown from the same ungraphed run (kinds on the side
        # stream overlap the others, so the entries may sum past ms_per_step)
        for kind in xss.PROF_KINDS:
            k_ms, k_n = xss.prof_read(kind)
            if k_n:
                kernels[kind] = {"ms_per_step": k_ms, "launches_per_step": k_n,
                                 "from": "one run without graph replay"}
    xss.prof_enable(False)
    xss.stream_status(stream.cuda_stream)
    checked = wl.check()
    percall = None
    if (hasattr(wl, "run_percall") and getattr(wl, "has_percall", True)
            and percall_segments is not None):
        percall = wl.percall_leg(percall_segments)

    if dist is not None:
        total_ms = max_over_ranks(total_ms, dist, "cuda")

    ms_per_step = total_ms / steps
    value = replica_throughput(n, ms_per_step, world)

    peak, peak_src = _peaks()
    active = dom_launches / dom_steps if dom_launches else 0
    avg_pass_ms = dom_ms / dom_launches if dom_launches else float("nan")
    achieved = wl.bytes_per_pass() / (avg_pass_ms / 1e3) / 1e9 if dom_launches else None
    kernel_name = "onesweep radix pass"
    if wl.dominant is None:
        # select: several short kernels; the roofline covers the whole operation
        kernel_name = getattr(wl, "roofline_name", "select (all kernels of one call)")
        avg_pass_ms = ms_per_step
        achieved = wl.bytes_model() / (ms_per_step / 1e3) / 1e9
        active = launches / steps
    traffic = _traffic(workload, n, n_full)

    e2e = None
    if do_e2e and rank == 0 and hasattr(wl, "host_run"):
        wl.host_setup()
        # the same W warm-up steps as the device leg
        for _ in range(max(warmup, 3)):
            wl.host_restore()
            wl.host_run()
        t = 0.0
        for _ in range(steps):
            wl.host_restore()
            t0 = time.perf_counter()
            wl.host_run()
            t += time.perf_counter() - t0
        bi, bo = wl.host_bytes()
        e2e = {"value": n * steps / t / 1e9, "unit": "Gkeys/s", "h2d_bytes_per_step": bi,
               "d2h_bytes_per_step": bo, "ms_per_step": t / steps * 1e3}
        if hasattr(wl, "host_check"):
            e2e["checked"] = bool(wl.host_check())   # the last step's host result

    cpu = None
    if rank == 0 and world == 1 and do_cpu:
        cpu = cpu_baseline(wl, sample_n=args.cpu_sample)

    # a published reference number for this exact workload (object_point3d only)
    published = (getattr(wl, "published", None) or {}).get(n)
    line = {
        "metric": "Gkeys/s", "value": value, "unit": "Gkeys/s", "n_gpus": world,
        "steps": steps, "warmup": warmup, "ms_per_step": ms_per_step,
        "higher_is_better": True, "scaling": "weak",
        "vs_baseline": value / published if published else None,
        **({"baseline_published": {"value": published, "unit": "Gkeys/s",
                                   "source": wl.published_source}} if published else {}),
        "dtype": DTYPE_OF[workload],
        "data": "synthetic (seeded, generated on device)",
        "config": {**wl.describe(), "parallelism": f"replicas x{world}"},
        "roofline": {"bound": "hbm", "kernel": kernel_name,
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "peak_source": peak_src,
                     "alg_bytes_per_launch": wl.bytes_per_pass(),
                     "avg_launch_ms": avg_pass_ms, "launches_per_step": active,
                     "traffic": traffic,
                     "sort_model_bytes": wl.bytes_model(),
                     "sort_frac": wl.bytes_model() / (ms_per_step / 1e3) / 1e9 / peak},
        "e2e": e2e,
        "cpu_baseline": cpu,
        "gpu_launches": launches,
        "kernels": kernels,
        "clocks": clk,
        "checked": checked,
        **({"percall": percall, "speedup_vs_percall": percall["ms_scaled"] / ms_per_step}
           if percall else {}),
        "wall_s_timed_region": wall,
    }
    wl.release()
    del wl
    torch.cuda.synchronize()
    torch.cuda.empty_cache()
    return {"line": line}


def measure_extras(args, ctx):
    """The other parts of the headline metric, each measured in the same run
    with its own clock record and check: float32 qsort at 2^28 (Gkeys/s and %
    of the HBM roofline), the literal config-4 batch against per-segment calls
    of the plain GPU sort (per-call leg over a contiguous sample of the
    segments, scaled by segment count), and a short serving run (p50/p99)."""
    out = {}
    steps, warmup = args.steps, max(args.warmup, 3)
    f32 = measure(args, ctx, "qsort_f32", 0, steps, warmup, do_e2e=False, do_cpu=False)["line"]
    out["qsort_f32_2e28"] = {k: f32[k] for k in ("value", "unit", "ms_per_step", "roofline",
                                                 "kernels", "clocks", "checked", "config")}
    seg_steps = max(3, min(steps, 5))
    seg = measure(args, ctx, "segmented", 0, seg_steps, 3, do_e2e=False, do_cpu=False,
                  percall_segments=args.percall_segments)["line"]
    out["segmented_config4"] = {k: seg.get(k) for k in (
        "value", "unit", "ms_per_step", "steps", "percall", "speedup_vs_percall", "roofline",
        "clocks", "checked", "config")}
    out["serving"] = serving_line(args, duration=args.extras_serving_s)
    return out


if __name__ == "__main__":
    main()

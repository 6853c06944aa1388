#!/usr/bin/env python3
"""Benchmark of the GB300 batched big-integer library.

Headline workload (one "step"): the batched add + signed-sub sweep over u64
limbs at 2^10 .. 2^18 bits, each size filling 2^27 limbs per operand (1 GiB),
80 % uniform and 20 % carry-chain instances -- 9 sizes x {add, sub} = 18
kernel launches per step.  The metric is the reference's add bandwidth,
GB/s = 3 * n * m * 8 / t (thesis/sections/performance.tex:75-78), over the
whole step (plus one sign byte per subtraction).  Operands are 1 GiB each,
far larger than the 129 MB L2, so no L2 flush is needed between launches.

  * value        -- device-resident inputs, whole-job GB/s over all ranks;
  * e2e          -- the same sweep through the host C-ABI entry points
                    (bi_host_add_u64 / bi_host_sub_u64) from pinned host
                    memory, copies in and out inside the timed region;
  * roofline     -- the add/sub kernel's algorithmic bytes per launch over
                    its CUDA-event launch time, against the measured HBM copy
                    peak (MEASURED_PEAKS.json), with the ncu DRAM traffic;
  * cpu_baseline -- the CPU oracle port on all host cores, full-size inputs;
  * extra        -- the multiply and division workloads (instances/s, word
                    products/s against the measured integer-pipe peak).

`--impl reference` times the reference's CPU implementation of the path on
the host cores -- the oracle port of it, all threads -- on the same metric
and workload, and prints the same JSON line with "impl": "reference".

Multi-GPU: instances are independent, so N ranks run N replicas of the step
(weak scaling, no collective on the data path; NCCL only carries the barrier
and the max over ranks of the elapsed time).

`--workload add|sub|mul|mul2048|div|divsweep|batch|serve` with `--bits`, `--total-limbs-log2`,
`--mul-m`, `--div-m`, `--batch-n` runs one operation on one size, or the
uneven batch, alone (used for profiling).
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "big-int_gb300"))

SEED_ADDSUB = 1001
BITS = [1 << k for k in range(10, 19)]
PUBLISHED_ADD_U64_GBS = 165.0     # mean C-V3 u64 add over 2^10..2^18 bits, GTX 1650 SUPER
FALLBACK_HBM_GBS = 6800.0


# ---------------------------------------------------------------------------
# clocks during the timed region (read-only NVML queries, nvidia-smi fallback)
# ---------------------------------------------------------------------------

class ClockSampler:
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}

    def __init__(self, period_s: float = 0.01):
        self.period = period_s
        self.samples = []
        self.stop_evt = threading.Event()
        self.nvml = None
        self.handle = None
        try:
            import torch

            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                raise RuntimeError("nvmlInit")
            h = ctypes.c_void_p()
            props = torch.cuda.get_device_properties(torch.cuda.current_device())
            bus = getattr(props, "pci_bus_id", None)
            ok = False
            if bus is not None:
                busid = f"{getattr(props, 'pci_domain_id', 0):08X}:{bus:02X}:{getattr(props, 'pci_device_id', 0):02X}.0"
                ok = nv.nvmlDeviceGetHandleByPciBusId_v2(busid.encode(), ctypes.byref(h)) == 0
            if not ok:
                ok = nv.nvmlDeviceGetHandleByIndex_v2(0, ctypes.byref(h)) == 0
            if ok:
                self.nvml, self.handle = nv, h
        except Exception:
            self.nvml = None

    def _sample_nvml(self):
        nv, h = self.nvml, self.handle
        sm, mx = ctypes.c_uint(), ctypes.c_uint()
        reasons = ctypes.c_ulonglong()
        nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(sm))
        nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx))
        f = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or nv.nvmlDeviceGetCurrentClocksThrottleReasons
        f(h, ctypes.byref(reasons))
        return sm.value, mx.value, reasons.value

    def _loop(self):
        while not self.stop_evt.is_set():
            try:
                self.samples.append(self._sample_nvml())
            except Exception:
                break
            time.sleep(self.period)

    def __enter__(self):
        if self.nvml is not None:
            self.thread = threading.Thread(target=self._loop, daemon=True)
            self.thread.start()
        else:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm,clocks_event_reasons.active",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        return self

    def __exit__(self, *exc):
        if self.nvml is not None:
            self.stop_evt.set()
            self.thread.join(timeout=2)
        else:
            self.proc.terminate()
            out, _ = self.proc.communicate(timeout=5)
            for line in out.splitlines():
                f = [x.strip() for x in line.split(",")]
                try:
                    self.samples.append((float(f[0]), float(f[1]), int(f[2], 16)))
                except Exception:
                    pass

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [s[0] for s in self.samples]
        reasons = set()
        for _, _, r in self.samples:
            for bit, name in self.REASONS.items():
                if r & bit:
                    reasons.add(name)
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(s[1] for s in self.samples)),
                "reasons": sorted(reasons), "samples": len(self.samples),
                "source": "nvml" if self.nvml is not None else "nvidia-smi"}


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(name: str):
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            return json.load(f).get(name)
    except Exception:
        return None


# ---------------------------------------------------------------------------
# helpers
# ---------------------------------------------------------------------------

def event_time(stream, fn, reps: int, warmup: int = 2):
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def graph_time(fn_on, reps: int = 20):
    """ms per call of fn_on(stream_handle) from one replay of a CUDA graph of
    `reps` captured calls: for launches short enough that the host's per-call
    overhead would otherwise set the interval."""
    import torch

    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        for _ in range(2):
            fn_on(int(s.cuda_stream))
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        for _ in range(reps):
            fn_on(int(s.cuda_stream))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(s):             # replay() launches on the current stream
        g.replay()
        torch.cuda.synchronize()
        e0.record(s)
        g.replay()
        e1.record(s)
    torch.cuda.synchronize()
    del g
    return e0.elapsed_time(e1) / reps


def whole_job(elapsed_ms: float, per_step_bytes: int, steps: int, world: int, device="cpu"):
    """(max over ranks of the timed region in ms, whole-job GB/s): every rank
    runs the full workload on its own GPU (weak scaling, no data exchange), so
    the job moves world x the per-rank bytes in the slowest rank's time."""
    import torch
    import torch.distributed as dist

    t = torch.tensor([float(elapsed_ms)], dtype=torch.float64, device=device)
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    ms = float(t.item())
    return ms, per_step_bytes * steps * world / (ms / 1e3) / 1e9


def check(L, st):
    if st != 0:
        raise RuntimeError(f"library call failed: {L.bi_last_error().decode()}")


def cpu_addsub(op: str, a: np.ndarray, b: np.ndarray, nthreads: int) -> float:
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O

    t0 = time.perf_counter()
    if op == "add":
        O.add(a, b, nthreads=nthreads)
    else:
        O.sub(a, b, nthreads=nthreads)
    return time.perf_counter() - t0


# Samples of the multiply and division workloads for the CPU timing beside
# them (a bounded slice of each GPU workload, about 0.1-0.4 s on 16 cores).
CPU_MUL_SAMPLE = {64: 32768, 256: 4096, 1024: 256, 2048: 64}
CPU_DIV_SAMPLE = {4: 65536, 16: 16384, 64: 2048, 256: 128, 1024: 8}


def cpu_sample_rate(fn, n: int) -> float:
    """Instances/s of fn() over n instances on the host (oracle port)."""
    t0 = time.perf_counter()
    fn()
    return n / (time.perf_counter() - t0)


# ---------------------------------------------------------------------------
# reference arm: the reference's CPU implementation (oracle port), host cores
# ---------------------------------------------------------------------------

def run_reference(args) -> None:
    if int(os.environ.get("RANK", "0")) != 0:
        return
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    from bigint_gb300.workloads import addsub_u64

    O.build()
    cores = os.cpu_count() or 1
    total = 1 << args.total_limbs_log2
    # the full workload, one (size, op) at a time so that host memory holds
    # one pair of 2^27-limb operands: generate (untimed), warm up, time K steps
    per_step = 0
    wall = 0.0
    for bits in BITS:
        for op in ("add", "sub"):
            a, b = addsub_u64(bits, seed=SEED_ADDSUB, total_limbs=total, op=op)
            per_step += 3 * a.size * 8 + (a.shape[0] if op == "sub" else 0)
            for _ in range(args.warmup):
                cpu_addsub(op, a, b, cores)
            for _ in range(args.steps):
                wall += cpu_addsub(op, a, b, cores)
            del a, b
    v = per_step * args.steps / wall / 1e9
    line = {
        "impl": "reference",
        "metric": "add/sub sweep GB/s (u64, 2^10..2^18 bits, 2^27 limbs per operand)",
        "value": round(v, 3), "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * wall / max(1, args.steps), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (splitmix64 seed 1001; 20% carry-chain instances)",
        "config": {"workload": "addsub_u64 sweep: 9 sizes 2^10..2^18 bits x {add, sub}, n = 2^27/m instances per size",
                   "sample": f"the full workload: 2^{args.total_limbs_log2} limbs per operand per size",
                   "same_config": args.total_limbs_log2 == 27},
        "cpu_baseline": {"value": round(v, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": "each step: the 9-size add+sub sweep at the GPU workload's full size; "
                                   "the oracle port of ker-add.cu.h / sub.fut, one pthread per core"},
        "e2e": {"value": round(v, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU measurements
# ---------------------------------------------------------------------------

def div_method(mv: int, n: int, sms: int) -> str:
    """The method bi_div_u64 picks for n divisions by mv-limb divisors
    (div_small_on_groups and div_use_long in divsmall.cuh): long division on
    one thread or one lane group (8, 16 or 32 lanes) per instance, or the
    shifted inverse on one CTA per instance."""
    if mv <= 16:
        return "long_group" if mv > 8 and n <= 48 * sms else "long_thread"
    if mv <= 64:
        return "long_group"
    if mv <= 1024 and n > (2 if mv <= 128 else 3 if mv <= 256 else 5 if mv <= 512 else 4) * sms:
        return "long_group"
    return "shinv"


def gu32ops(n: int, words: int, ms: float) -> float:
    """The reference's own multiply rate, "Gu32ops" (cuda/main.cu:393-400):
    300 M log2(M) u32 operations per instance of an M-word (u32) product,
    FFT-normalised (a count for comparison with FFT multiplies, not work
    done), in Gops/s.  M is the product's size in u32 words."""
    return n * 300 * words * (words.bit_length() - 1) / (ms * 1e6)


def long_div_limb_products(mu: int, mv: int) -> int:
    """64x64-bit limb products of schoolbook long division of a mu-limb
    dividend by an mv-limb divisor with a nonzero top limb: one q-hat * v row
    per quotient limb (the estimates' own products are not counted)."""
    return (mu - mv + 1) * mv


def div_limb_products(mu: int, mv: int) -> int:
    """64x64-bit limb products in the multiplications one division performs
    (the shifted-inverse division of divcore.cuh on a mu-limb dividend and an
    mv-limb divisor, both normalised to full length): the Newton steps'
    low product V*Y mod B^(s+1) and short product Y*|E| (columns >= 2p-1),
    the quotient's short product u*Y (columns >= P+K-2) and the low product
    q*v mod B^(K+1)."""
    def pairs(la, lb, lo, hi):
        n = 0
        for c in range(max(lo, 0), hi):
            i0, i1 = max(0, c - lb + 1), min(la - 1, c)
            if i1 >= i0:
                n += i1 - i0 + 1
        return n

    K, H = mv, mu
    Qlen = H - K + 1
    P = Qlen + 1
    sched, x = [P], P
    while x > 2:
        x = (x + 2) // 2
        sched.append(x)
    total, p = 0, 1
    for pn in reversed(sched):
        if pn <= p:
            continue
        sl = pn + 1
        total += pairs(sl, p + 1, 0, sl + 1)
        total += pairs(p + 1, sl + 1, (2 * p - 1) // 8 * 8, p + sl + 2)
        p = pn
    total += pairs(H, P + 1, (P + K - 2) // 8 * 8, H + P + 1)
    total += pairs(Qlen + 1, K, 0, K + 1)
    return total


def measure_extra(B, L, stream, args):
    """Multiply and division workloads: instances/s and word-product rates."""
    import torch

    from bigint_gb300.workloads import MUL_U64, device_uniform_u64, mul2048_u32, mul_u64_device

    sp = int(stream.cuda_stream)
    rates = B.probe_intpipe()
    peak_wps = max(rates.values())
    peak_gbs = measured_peaks()[0]
    out = {"intpipe_peak_word_products_per_s": peak_wps,
           "intpipe_peak_form": max(rates, key=rates.get)}
    mul = {}
    for m, n in MUL_U64:
        a, b = mul_u64_device(m, n)
        r = torch.empty((n, 2 * m), dtype=torch.int64, device="cuda")
        ms = event_time(stream, lambda: check(L, L.bi_mulfull_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, sp)), 5)
        rt = torch.empty((n, m), dtype=torch.int64, device="cuda")
        ms_t = event_time(stream, lambda: check(L, L.bi_mul_u64(a.data_ptr(), b.data_ptr(), rt.data_ptr(), m, n, sp)), 5)
        wp = n * (2 * m) ** 2
        # the same calls after the autotuner picked the tiling on these operands
        chosen = (ctypes.c_int * 2)()
        check(L, L.bi_mul_autotune_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, 1, 3,
                                       ctypes.cast(chosen, ctypes.c_void_p), sp))
        ms_tuned = event_time(stream, lambda: check(L, L.bi_mulfull_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n,
                                                                         sp)), 5)
        check(L, L.bi_mul_set_tuning_u64(m, 1, 0, 0))       # back to the library's own choice
        cpu = None
        if not args.no_cpu:
            sys.path.insert(0, os.path.join(REPO, "oracle"))
            import oracle as O

            k = CPU_MUL_SAMPLE.get(m, 64)
            ha, hb = B.to_host(a[:k], np.uint64), B.to_host(b[:k], np.uint64)
            th = os.cpu_count() or 1
            cpu = {"instances_per_s": round(cpu_sample_rate(lambda: O.mulfull(ha, hb, nthreads=th), k)),
                   "threads": th, "sample": f"the first {k} pairs", "kind": "port",
                   "what": "the oracle's C schoolbook full product (stands in for the reference's mult.c prototype)"}
        mul[f"m{m}_n{n}"] = {"full_instances_per_s": round(n / ms * 1e3), "full_ms": round(ms, 4), "cpu": cpu,
                             "word_products_per_s": wp / ms * 1e3, "frac_of_intpipe_peak": round(wp / ms * 1e3 / peak_wps, 4),
                             # the reference's FFT-normalised figure: its full product is a 2m-limb
                             # (4m-word) truncated launch on zero-padded operands
                             "full_gu32ops_fft_normalised": round(gu32ops(n, 4 * m, ms), 1),
                             "truncated_instances_per_s": round(n / ms_t * 1e3), "truncated_ms": round(ms_t, 4),
                             "truncated_gu32ops_fft_normalised": round(gu32ops(n, 2 * m, ms_t), 1),
                             "autotuned_full_instances_per_s": round(n / ms_tuned * 1e3),
                             "autotuned_frac_of_intpipe_peak": round(wp / ms_tuned * 1e3 / peak_wps, 4),
                             "autotuned_tiling": {"instances_per_cta": chosen[0], "row_slices": chosen[1]}}
        del a, b, r, rt
    out["mul_u64_full"] = mul
    a, b = mul2048_u32()
    da, db = B.to_device(a), B.to_device(b)
    r = torch.empty((a.shape[0], 128), dtype=torch.int32, device="cuda")
    ms = graph_time(lambda st: check(L, L.bi_mulfull_u32(da.data_ptr(), db.data_ptr(), r.data_ptr(), 64, 4096, st)))
    ms_ev = event_time(stream, lambda: check(L, L.bi_mulfull_u32(da.data_ptr(), db.data_ptr(), r.data_ptr(), 64, 4096, sp)), 20)
    out["mul2048_u32"] = {"instances_per_s": round(4096 / ms * 1e3), "ms": round(ms, 5),
                          "instances_per_s_python_launches": round(4096 / ms_ev * 1e3),
                          "note": "4096 pairs of 64 u32 limbs, 10% all-ones, full 128-limb product; a launch this "
                                  "short is timed as one replay of a CUDA graph of 20 launches (host overhead "
                                  "excluded, as for the reference kernel beside it)"}
    # small full products (the thread and warp kernels): 2^22 limbs of input per operand and size, graph-timed
    small = {}
    for m in (2, 4, 8, 16, 32):
        n = (1 << 22) // m
        a = device_uniform_u64(31, n, m)
        b = device_uniform_u64(32, n, m)
        r = torch.empty((n, 2 * m), dtype=torch.int64, device="cuda")
        ms = graph_time(lambda st: check(L, L.bi_mulfull_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, st)), 5)
        wp = n * (2 * m) ** 2
        # the truncated product (mod B^m, the reference's convMul semantics): m(m+1)/2 limb products
        rt = torch.empty((n, m), dtype=torch.int64, device="cuda")
        ms_t = graph_time(lambda st: check(L, L.bi_mul_u64(a.data_ptr(), b.data_ptr(), rt.data_ptr(), m, n, st)), 5)
        wp_t = n * 4 * m * (m + 1) // 2
        # the autotuner weighs the thread and warp kernels against the CTA tilings (64-bit limbs)
        chosen = (ctypes.c_int * 2)()
        check(L, L.bi_mul_autotune_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, 1, 3,
                                       ctypes.cast(chosen, ctypes.c_void_p), sp))
        ms_tuned = graph_time(lambda st: check(L, L.bi_mulfull_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n,
                                                                    st)), 5)
        check(L, L.bi_mul_set_tuning_u64(m, 1, 0, 0))       # back to the library's own choice
        pick = ("warp kernel, 32-bit words" if (chosen[0], chosen[1]) == (0, 0) else
                "thread kernel, 64-bit limbs" if (chosen[0], chosen[1]) == (0, 1) else
                f"CTA kernel, 64-bit limbs, {chosen[0]} instances x {chosen[1]} slices")
        small[f"m{m}_n{n}"] = {"instances_per_s": round(n / ms * 1e3), "word_products_per_s": wp / ms * 1e3,
                               "frac_of_intpipe_peak": round(wp / ms * 1e3 / peak_wps, 4),
                               "truncated_instances_per_s": round(n / ms_t * 1e3),
                               "truncated_frac_of_intpipe_peak": round(wp_t / ms_t * 1e3 / peak_wps, 4),
                               "autotuned_instances_per_s": round(n / ms_tuned * 1e3), "autotuned_pick": pick}
        del a, b, r, rt
    out["mulfull_u64_small"] = small
    div = {}
    # 2^23 dividend limbs a size: dividends, divisors, quotients and remainders (192 MB) pass
    # the 129 MB L2, so the small sizes are timed on memory, not on one ~10 us launch
    # 384 and 768: divisors between the powers of two, on the 24-limb-a-lane shapes
    for mv, n in [(4, 1 << 20), (16, 1 << 18), (64, 1 << 16), (256, 1 << 14), (384, (1 << 23) // 768),
                  (768, (1 << 23) // 1536), (1024, 1 << 12)]:
        u = device_uniform_u64(11, n, 2 * mv)
        v = device_uniform_u64(12, n, mv)
        v[:, -1] |= 1
        q = torch.empty_like(u)
        rr = torch.empty_like(v)
        st = torch.empty(n, dtype=torch.uint8, device="cuda")
        # one replay of a CUDA graph of the calls: the shortest divisions take ~10 us, which
        # the host's per-call overhead would otherwise set
        ms = graph_time(lambda s_: check(L, L.bi_div_u64(u.data_ptr(), v.data_ptr(), q.data_ptr(), rr.data_ptr(),
                                                           st.data_ptr(), 2 * mv, mv, n, s_)), 5)
        ms_shinv = graph_time(lambda s_: check(L, L.bi_div_shinv_u64(u.data_ptr(), v.data_ptr(), q.data_ptr(),
                                                                       rr.data_ptr(), st.data_ptr(), 2 * mv, mv, n,
                                                                       s_)), 5)
        method = div_method(mv, n, torch.cuda.get_device_properties(0).multi_processor_count)
        # 32x32-bit word products per division of the method that ran
        wp = 4 * (div_limb_products(2 * mv, mv) if method == "shinv" else long_div_limb_products(2 * mv, mv))
        cpu = None
        if not args.no_cpu:
            sys.path.insert(0, os.path.join(REPO, "oracle"))
            import oracle as O

            k = CPU_DIV_SAMPLE.get(mv, 8)
            hu = B.to_host(u[:k], np.uint64).view(np.uint32)
            hv = np.zeros((k, 4 * mv), np.uint32)       # div.c divides equal sizes: v zero-extended
            hv[:, : 2 * mv] = B.to_host(v[:k], np.uint64).view(np.uint32)
            th = os.cpu_count() or 1
            cpu = {"instances_per_s": round(cpu_sample_rate(lambda: O.div_ref(hu, hv, nthreads=th), k)),
                   "threads": th, "sample": f"the first {k} pairs", "kind": "port",
                   "what": "the oracle's restatement of prototypes/div.c div_shinv (u32 digits), all host threads"}
        # bytes a division moves: u and v read, q (as many limbs as u), r and a status byte written
        by = n * (2 * (2 * mv) * 8 + 2 * mv * 8 + 1)
        entry = {"method": method, "instances_per_s": round(n / ms * 1e3), "ms": round(ms, 4), "cpu": cpu,
                 "word_products_per_div": wp, "word_products_per_s": wp * n / ms * 1e3,
                 "frac_of_intpipe_peak": round(wp * n / ms * 1e3 / peak_wps, 4),
                 "GBps": round(by / ms / 1e6), "frac_of_hbm_peak": round(by / ms * 1e3 / (peak_gbs * 1e9), 4),
                 "shinv_instances_per_s": round(n / ms_shinv * 1e3)}
        if not args.no_cpu:
            # the reference's own work figure: the word products of div.c's multiplications on this
            # instance (the first pair), as the instrumented oracle counts them; the rate in that
            # work can exceed the integer peak because long division does far fewer products
            divc = O.div_ref_word_products(hu[0], hv[0])
            entry["divc_word_products_per_div"] = divc
            entry["intpipe_peak_multiple_in_divc_work"] = round(divc * n / ms * 1e3 / peak_wps, 3)
        div[f"m{mv}_n{n}"] = entry
        del u, v, q, rr, st
    out["div_u64_2m_by_m"] = div
    out["uneven_batch"] = measure_uneven_batch(B, L, stream, peak_wps=peak_wps)
    out["reference_cuda_kernels"] = measure_reference_kernels(B, L, stream)
    out["chains"] = measure_chains(B, L, stream)
    out["serving"] = measure_serving(B)
    torch.cuda.empty_cache()
    return out


def measure_uneven_batch(B, L, stream, n: int = 100_000, peak_wps: float = 0.0):
    """100k mixed instances (sizes log-uniform 256..65536 bits; 20% add, 20% sub,
    40% full multiply, 20% division): one graph-captured plan launch versus the
    plain one-launch-per-(op, size) kernels on the same instances."""
    import torch

    d, arena, out_limbs, nflags = B.workloads.uneven_batch(n=n)
    din = B.to_device(arena)
    dout = torch.zeros(out_limbs, dtype=torch.int64, device="cuda")
    dfl = torch.zeros(nflags, dtype=torch.uint8, device="cuda")
    t0 = time.perf_counter()
    plan = B.Plan(d, len(arena), out_limbs, nflags)
    plan_ms = (time.perf_counter() - t0) * 1e3
    chosen = plan.autotune(din, dout, dfl, reps=2)
    ms_batch = event_time(stream, lambda: plan.execute(din, dout, dfl, stream=stream), 5, 2)
    # plain per-size launches: operands regrouped per (op, m) (untimed), one launch per group
    sp = int(stream.cuda_stream)
    groups = {}
    for i, key in enumerate(zip(d["op"].tolist(), d["m"].tolist(), d["mb"].tolist())):
        groups.setdefault(key, []).append(i)
    calls = []
    for (op, m, mb), idx in groups.items():
        idx = np.asarray(idx)
        ia = torch.from_numpy((d["a"][idx][:, None] + np.arange(m)[None, :]).astype(np.int64)).cuda()
        ib = torch.from_numpy((d["b"][idx][:, None] + np.arange(mb)[None, :]).astype(np.int64)).cuda()
        a, b = din[ia].contiguous(), din[ib].contiguous()
        g = len(idx)
        if op in (B.OP_ADD, B.OP_SUB):
            r = torch.empty_like(a)
            s = torch.empty(g, dtype=torch.uint8, device="cuda")
            calls.append((op, a, b, r, s, m, mb, g))
        elif op == B.OP_MULFULL:
            calls.append((op, a, b, torch.empty((g, 2 * m), dtype=torch.int64, device="cuda"), None, m, mb, g))
        else:
            calls.append((op, a, b, (torch.empty_like(a), torch.empty_like(b)),
                          torch.empty(g, dtype=torch.uint8, device="cuda"), m, mb, g))

    def per_size_on(s_):
        for op, a, b, r, s, m, mb, g in calls:
            if op == B.OP_ADD:
                check(L, L.bi_add_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, g, s_))
            elif op == B.OP_SUB:
                check(L, L.bi_sub_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), s.data_ptr(), m, g, s_))
            elif op == B.OP_MULFULL:
                check(L, L.bi_mulfull_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, g, s_))
            else:
                check(L, L.bi_div_u64(a.data_ptr(), b.data_ptr(), r[0].data_ptr(), r[1].data_ptr(), s.data_ptr(),
                                      m, mb, g, s_))

    ms_per_size = event_time(stream, lambda: per_size_on(sp), 2, 1)
    # the same launches captured once into a CUDA graph and replayed: the
    # per-size baseline without the host's per-call overhead
    ms_per_size_graph = graph_time(per_size_on, reps=1)
    st = plan.stats()
    plan.close()
    # the batch's algorithmic work: word products of the full multiplies (4 m^2)
    # and of long division ((m - mb + 1) mb limb products, 4 words each), and the
    # bytes of add/sub (read a, b, write r; + 1 sign byte for sub)
    ops, ms_, mbs = d["op"].astype(np.int64), d["m"].astype(np.int64), d["mb"].astype(np.int64)
    wp = int((4 * ms_ * ms_)[ops == B.OP_MULFULL].sum() + (4 * ms_ * ms_)[ops == B.OP_MUL].sum() // 2
             + (4 * (ms_ - mbs + 1) * mbs)[ops == B.OP_DIV].sum())
    ab = int((24 * ms_)[ops == B.OP_ADD].sum() + (24 * ms_ + 1)[ops == B.OP_SUB].sum())
    ipeak = peak_wps or max(B.probe_intpipe().values())
    hpeak, _ = measured_peaks()
    f_int = wp / (ms_batch / 1e3) / ipeak
    f_hbm = ab / (ms_batch / 1e3) / 1e9 / hpeak
    del din, dout, dfl, calls
    torch.cuda.empty_cache()
    return {"instances": n, "batched_inst_per_s": round(n / ms_batch * 1e3), "batched_ms": round(ms_batch, 3),
            "per_size_launch_inst_per_s": round(n / ms_per_size * 1e3), "per_size_launch_ms": round(ms_per_size, 3),
            "per_size_graph_inst_per_s": round(n / ms_per_size_graph * 1e3),
            "per_size_graph_ms": round(ms_per_size_graph, 3),
            "speedup_vs_per_size_launch": round(ms_per_size / ms_batch, 2),
            "speedup_vs_per_size_graph": round(ms_per_size_graph / ms_batch, 2),
            "per_size_launches": len(groups),
            "roofline": {"word_products": wp, "addsub_bytes": ab,
                         "word_products_per_s": wp / (ms_batch / 1e3), "frac_of_intpipe_peak": round(f_int, 4),
                         "addsub_gbs": round(ab / (ms_batch / 1e3) / 1e9, 1), "frac_of_hbm_peak": round(f_hbm, 4),
                         "sum_of_fracs": round(f_int + f_hbm, 4),
                         "note": "the batch's kernels share the GPU: the two fractions of the one replay time add up "
                                 "to the share of the machine's integer-pipe and HBM peaks the batch uses"},
            "plan_create_ms": round(plan_ms, 1), "autotune": chosen, "plan": st,
            "note": "one CUDA-graph replay of the plan's concurrent persistent kernels vs one plain launch per "
                    "(op, m) group, issued from Python and as one replay of those launches captured in a CUDA graph"}


def measure_serving(B, rates=None, seconds: float = 0.2, max_requests: int = 100_000, streams: int = 4,
                    saturation_rates=(2_000_000, 4_000_000)):
    """Poisson streams of requests (sizes log-uniform 512..32768 bits; 15% add,
    15% sub, 40% full multiply, 30% division; operands resident in a 2^24-limb
    device pool; a 2^26-limb result arena as the HBM budget): the
    device-resident loop versus one library launch per request round-robin
    over `streams` streams.  Latency runs from a request's arrival to the
    host seeing its completion."""
    import torch

    from bigint_gb300.workloads import SERVE_RATES, serve_pool_device, serve_stream

    pool_limbs = 1 << 24
    _, _, pool_seed = serve_stream(1, 1.0, pool_limbs=pool_limbs)
    pool = serve_pool_device(pool_limbs, pool_seed)
    arena = torch.empty(1 << 26, dtype=torch.int64, device="cuda")
    torch.cuda.synchronize()
    rates = rates or SERVE_RATES
    streams_of = {r: serve_stream(int(min(max_requests, max(2000, r * seconds))), r, pool_limbs=pool_limbs)
                  for r in rates}
    warm = serve_stream(2000, 100_000, seed=9, pool_limbs=pool_limbs)
    keep = ("requests", "launches", "busy", "achieved_rps", "offered_rps", "p50_us", "p90_us", "p99_us",
            "p999_us", "max_us", "mean_us")

    def short(rep):
        return {k: (round(rep[k], 2) if isinstance(rep[k], float) else rep[k]) for k in keep}

    def per_class(d, lat_ns):
        """p50 / p99 latency (us) and count per (op, operand limbs) class."""
        lat = lat_ns.astype(np.float64) / 1e3
        names = {B.OP_ADD: "add", B.OP_SUB: "sub", B.OP_MULFULL: "mulfull", B.OP_DIV: "div"}
        res = {}
        for op, name in names.items():
            for lo, hi in ((1, 64), (65, 256), (257, 512)):
                sel = (d["op"] == op) & (d["m"] >= lo) & (d["m"] <= hi)
                if sel.sum() >= 20:
                    x = lat[sel]
                    res[f"{name}_m{lo}-{hi}"] = [int(sel.sum()), round(float(np.percentile(x, 50)), 1),
                                                 round(float(np.percentile(x, 99)), 1)]
        return res

    out = {}
    beyond = {}
    with B.Server(pool, arena) as srv:
        info = srv.info()
        srv.replay(warm[0], warm[1])
        for r in rates:
            d, arr, _ = streams_of[r]
            lat, _, rep = srv.replay(d, arr)
            out[str(r)] = {"loop": short(rep), "loop_per_class_n_p50_p99_us": per_class(d, lat)}
        # past the offered loads: where the loop saturates
        for r in saturation_rates:
            d, arr, _ = serve_stream(max_requests, r, seed=1005, pool_limbs=pool_limbs)
            _, _, rep = srv.replay(d, arr)
            beyond[str(r)] = short(rep)
    # the loop has stopped: the per-request launches get the whole GPU
    B.replay_plain(pool, arena, warm[0], warm[1], streams=streams)
    for r in rates:
        d, arr, _ = streams_of[r]
        lat, _, rep = B.replay_plain(pool, arena, d, arr, streams=streams)
        out[str(r)]["per_request_launch"] = short(rep)
        out[str(r)]["launch_per_class_n_p50_p99_us"] = per_class(d, lat)
        lo, pl = out[str(r)]["loop"], out[str(r)]["per_request_launch"]
        out[str(r)]["p99_ratio_launch_over_loop"] = round(pl["p99_us"] / lo["p99_us"], 2) if lo["p99_us"] else None
    del pool, arena
    torch.cuda.empty_cache()
    return {"rates_rps": out, "loop_beyond_offered_loads": beyond, "loop_ctas": info["ctas"],
            "loop_smem_bytes": info["smem_bytes"],
            "result_arena_limbs": info["arena_limbs"], "per_request_streams": streams,
            "note": "open-loop Poisson replay; latency = completion seen by the host - scheduled arrival"}


def measure_chains(B, L, stream):
    """The reference's second benchmark type: ten chained additions
    (add chain p = 10, GB/s as 3 n m 8 / time, intermediates on chip) and six
    chained truncated multiplications (mul chain p = 6), beside the
    reference's own baddKer3Bench / convMul5Bench on the same inputs."""
    import torch

    from bigint_gb300.workloads import addsub_u64_device, device_uniform_u64

    sys.path.insert(0, os.path.join(REPO, "baseline"))
    import refgpu

    R = refgpu.lib() if refgpu.build() else None
    sp = int(stream.cuda_stream)
    out = {"add10_u64_gbs": {}, "mul6_u64": {}}
    for m in refgpu.ADD10_SIZES:
        a, b = addsub_u64_device(m * 64, seed=SEED_ADDSUB, total_limbs=1 << 27, op="add")
        n = a.shape[0]
        r = torch.empty_like(a)
        ms = event_time(stream, lambda: check(L, L.bi_add_chain_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(),
                                                                     m, n, 10, sp)), 5)
        row = {"ours": round(3 * n * m * 8 / ms / 1e6, 1)}
        if R is not None:
            rr = torch.empty_like(a)
            # baddKer3Bench: the reference's fastest ten-addition kernel (same additions; its
            # in-place buffers drop the carries of steps 2..10, so its values differ)
            if R.ref_add10_u64(a.data_ptr(), b.data_ptr(), rr.data_ptr(), m, n, sp) == 0:
                ms_r = event_time(stream, lambda: R.ref_add10_u64(a.data_ptr(), b.data_ptr(), rr.data_ptr(), m, n,
                                                                  sp), 5)
                row["reference_baddKer3Bench"] = round(3 * n * m * 8 / ms_r / 1e6, 1)
            # baddKer1Bench computes 10(a+b): the values to match
            if m in refgpu.ADD10_V1_SIZES and R.ref_add10v1_u64(a.data_ptr(), b.data_ptr(), rr.data_ptr(), m, n,
                                                                sp) == 0:
                ms_1 = event_time(stream, lambda: R.ref_add10v1_u64(a.data_ptr(), b.data_ptr(), rr.data_ptr(), m,
                                                                    n, sp), 3)
                row["reference_baddKer1Bench"] = round(3 * n * m * 8 / ms_1 / 1e6, 1)
                row["bit_exact_vs_baddKer1Bench"] = bool((rr == r).all())
        out["add10_u64_gbs"][str(m * 64)] = row
        del a, b, r
    for m, n in [(64, 1 << 16), (256, 1 << 14), (1024, 1 << 12)]:
        a = device_uniform_u64(21, n, m)
        b = device_uniform_u64(22, n, m)
        r = torch.empty_like(a)
        ms = event_time(stream, lambda: check(L, L.bi_mul_chain_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(),
                                                                     m, n, 6, sp)), 5)
        wp = n * 6 * 4 * m * (m + 1) // 2          # six truncated products, 32x32-bit word products
        row = {"ours_inst_per_s": round(n / ms * 1e3), "ours_word_products_per_s": wp / ms * 1e3}
        if R is not None:
            rr = torch.empty_like(a)
            if R.ref_mul6_u64(a.data_ptr(), b.data_ptr(), rr.data_ptr(), m, n, sp) == 0:
                ms_r = event_time(stream, lambda: R.ref_mul6_u64(a.data_ptr(), b.data_ptr(), rr.data_ptr(), m, n,
                                                                 sp), 5)
                row["reference_convMul5Bench_inst_per_s"] = round(n / ms_r * 1e3)
                row["bit_exact"] = bool((rr == r).all())
        out["mul6_u64"][f"m{m}_n{n}"] = row
        del a, b, r
    torch.cuda.empty_cache()
    return out


def measure_reference_kernels(B, L, stream):
    """The reference's own kernels (baddKer3, convMul5) on the same GPU and inputs."""
    import torch

    from bigint_gb300.workloads import MUL_U64, addsub_u64_device, device_uniform_u64, mul2048_u32, mul_u64_device

    sys.path.insert(0, os.path.join(REPO, "baseline"))
    try:
        import refgpu

        if not refgpu.build() or refgpu.lib() is None:
            return {"unavailable": "reference kernel headers were not staged"}
    except Exception as e:  # a baseline only: never fail the bench on it
        return {"unavailable": f"reference kernels did not build: {e}"}
    R = refgpu.lib()
    sp = int(stream.cuda_stream)
    res = {"add_u64_gbs": {}, "mul_u64": {}}
    total = 1 << 27
    for bits in BITS:
        m = bits // 64
        a, b = addsub_u64_device(bits, seed=SEED_ADDSUB, total_limbs=total, op="add")
        n = a.shape[0]
        r = torch.empty_like(a)
        ms_ref = event_time(stream, lambda: R.ref_add_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, sp), 5)
        ms_ours = event_time(stream, lambda: check(L, L.bi_add_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, sp)), 5)
        res["add_u64_gbs"][str(bits)] = {"reference_baddKer3": round(3 * total * 8 / ms_ref / 1e6, 1),
                                          "ours": round(3 * total * 8 / ms_ours / 1e6, 1)}
        del a, b, r
    for m, n in MUL_U64:
        a, b = mul_u64_device(m, n)
        rt = torch.empty_like(a)
        ms_tr = event_time(stream, lambda: R.ref_mul_u64(a.data_ptr(), b.data_ptr(), rt.data_ptr(), m, n, sp), 3)
        ms_ours_tr = event_time(stream, lambda: check(L, L.bi_mul_u64(a.data_ptr(), b.data_ptr(), rt.data_ptr(), m, n, sp)), 3)
        entry = {"truncated_reference_inst_per_s": round(n / ms_tr * 1e3),
                 "truncated_ours_inst_per_s": round(n / ms_ours_tr * 1e3),
                 "truncated_reference_gu32ops_fft_normalised": round(gu32ops(n, 2 * m, ms_tr), 1),
                 "truncated_ours_gu32ops_fft_normalised": round(gu32ops(n, 2 * m, ms_ours_tr), 1)}
        if 2 * m in refgpu.MUL_SIZES_U64:
            pa = torch.zeros((n, 2 * m), dtype=torch.int64, device="cuda")
            pb = torch.zeros_like(pa)
            pa[:, :m] = a
            pb[:, :m] = b
            rf = torch.empty_like(pa)
            ms_f = event_time(stream, lambda: R.ref_mul_u64(pa.data_ptr(), pb.data_ptr(), rf.data_ptr(), 2 * m, n, sp), 3)
            ms_ours_f = event_time(stream, lambda: check(L, L.bi_mulfull_u64(a.data_ptr(), b.data_ptr(), rf.data_ptr(), m, n, sp)), 3)
            entry["full_reference_inst_per_s"] = round(n / ms_f * 1e3)
            entry["full_ours_inst_per_s"] = round(n / ms_ours_f * 1e3)
            entry["full_reference_gu32ops_fft_normalised"] = round(gu32ops(n, 4 * m, ms_f), 1)
            entry["full_ours_gu32ops_fft_normalised"] = round(gu32ops(n, 4 * m, ms_ours_f), 1)
            del pa, pb, rf
        else:
            entry["full_reference"] = "unavailable: convMul5 at 2m=%d limbs needs >48 KiB static shared memory" % (2 * m)
        res["mul_u64"][f"m{m}_n{n}"] = entry
        del a, b, rt
    # the small end of the reference's own multiply sweep (cuda/main.cu:511-512), 2^22 limbs an
    # operand: convMul5 at m (truncated) and at 2m on zero-padded inputs (full), graph-timed as both
    # are a few microseconds a launch
    res["mul_u64_small"] = {}
    for m in (16, 32):
        n = (1 << 22) // m
        a = device_uniform_u64(41, n, m)
        b = device_uniform_u64(42, n, m)
        rt = torch.empty_like(a)
        ms_tr = graph_time(lambda st: R.ref_mul_u64(a.data_ptr(), b.data_ptr(), rt.data_ptr(), m, n, st), 5)
        ms_ours_tr = graph_time(lambda st: check(L, L.bi_mul_u64(a.data_ptr(), b.data_ptr(), rt.data_ptr(), m, n,
                                                                 st)), 5)
        pa = torch.zeros((n, 2 * m), dtype=torch.int64, device="cuda")
        pb = torch.zeros_like(pa)
        pa[:, :m] = a
        pb[:, :m] = b
        rf = torch.empty_like(pa)
        ms_f = graph_time(lambda st: R.ref_mul_u64(pa.data_ptr(), pb.data_ptr(), rf.data_ptr(), 2 * m, n, st), 5)
        ms_ours_f = graph_time(lambda st: check(L, L.bi_mulfull_u64(a.data_ptr(), b.data_ptr(), rf.data_ptr(), m, n,
                                                                    st)), 5)
        res["mul_u64_small"][f"m{m}_n{n}"] = {
            "truncated_reference_inst_per_s": round(n / ms_tr * 1e3), "truncated_ours_inst_per_s": round(n / ms_ours_tr * 1e3),
            "full_reference_inst_per_s": round(n / ms_f * 1e3), "full_ours_inst_per_s": round(n / ms_ours_f * 1e3)}
        del a, b, rt, pa, pb, rf
    a, b = mul2048_u32()
    n, m = a.shape
    pa = np.zeros((n, 2 * m), np.uint32)
    pb = np.zeros((n, 2 * m), np.uint32)
    pa[:, :m] = a
    pb[:, :m] = b
    dpa, dpb = B.to_device(pa), B.to_device(pb)
    rf = torch.empty_like(dpa)
    ms_ref = graph_time(lambda st: R.ref_mul_u32(dpa.data_ptr(), dpb.data_ptr(), rf.data_ptr(), 2 * m, n, st))
    res["mul2048_u32_full_reference_inst_per_s"] = round(n / ms_ref * 1e3)
    return res


def run_single(args) -> None:
    """One operation on one size (for profiling); prints a small JSON line."""
    import torch

    import bigint_gb300 as B
    from bigint_gb300.workloads import addsub_u64_device, device_uniform_u64, mul_u64_device

    B.build()
    L = B.lib()
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    w = args.workload
    if w in ("add", "sub"):
        bits = args.bits or 65536
        a, b = addsub_u64_device(bits, seed=SEED_ADDSUB, total_limbs=1 << args.total_limbs_log2, op=w)
        n, m = a.shape
        r = torch.empty_like(a)
        s = torch.empty(n, dtype=torch.uint8, device="cuda")
        fn = (lambda: check(L, L.bi_add_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, sp))) if w == "add" else \
             (lambda: check(L, L.bi_sub_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), s.data_ptr(), m, n, sp)))
        ms = event_time(stream, fn, args.steps, args.warmup)
        print(json.dumps({"workload": w, "bits": bits, "n": n, "ms": ms, "GBps": 3 * n * m * 8 / ms / 1e6}))
    elif w == "mul":
        m = args.mul_m
        n = max(1, (1 << args.total_limbs_log2) // m)
        a, b = mul_u64_device(m, n)
        r = torch.empty((n, 2 * m), dtype=torch.int64, device="cuda")
        ms = event_time(stream, lambda: check(L, L.bi_mulfull_u64(a.data_ptr(), b.data_ptr(), r.data_ptr(), m, n, sp)),
                        args.steps, args.warmup)
        print(json.dumps({"workload": w, "m": m, "n": n, "ms": ms, "word_products_per_s": n * 4 * m * m / ms * 1e3}))
    elif w == "div":
        mv = args.div_m
        n = max(1, (1 << args.total_limbs_log2) // (2 * mv))
        u = device_uniform_u64(11, n, 2 * mv)
        v = device_uniform_u64(12, n, mv)
        v[:, -1] |= 1
        q, rr = torch.empty_like(u), torch.empty_like(v)
        st = torch.empty(n, dtype=torch.uint8, device="cuda")
        fn = L.bi_div_u64 if args.div_method == "auto" else getattr(L, f"bi_div_{args.div_method}_u64")
        ms = event_time(stream, lambda: check(L, fn(u.data_ptr(), v.data_ptr(), q.data_ptr(), rr.data_ptr(),
                                                    st.data_ptr(), 2 * mv, mv, n, sp)), args.steps, args.warmup)
        print(json.dumps({"workload": w, "m": mv, "n": n, "method": args.div_method, "ms": ms,
                          "instances_per_s": n / ms * 1e3}))
    elif w == "divsweep":
        # long division vs the shifted inverse over divisor sizes and batch sizes (2m/m)
        rows = {}
        for mv in (32, 64, 128, 256, 512, 1024):
            mu = 2 * mv
            for n in (1, 38, 152, 304, 608, 1216, 2432):
                u = device_uniform_u64(11, n, mu)
                v = device_uniform_u64(12, n, mv)
                v[:, -1] |= 1
                q, rr = torch.empty_like(u), torch.empty_like(v)
                st = torch.empty(n, dtype=torch.uint8, device="cuda")
                row = {}
                for name in ("bi_div_long_u64", "bi_div_shinv_u64"):
                    fn = getattr(L, name)
                    ms = event_time(stream, lambda: check(L, fn(u.data_ptr(), v.data_ptr(), q.data_ptr(), rr.data_ptr(),
                                                                st.data_ptr(), mu, mv, n, sp)), 5 if mv < 512 else 2)
                    row[name] = round(ms * 1e3, 1)
                rows[f"{mu}/{mv} n={n}"] = {"long_us": row["bi_div_long_u64"], "shinv_us": row["bi_div_shinv_u64"]}
        print(json.dumps({"workload": w, "us_per_call": rows}))
    elif w == "mul2048":
        from bigint_gb300.workloads import mul2048_u32

        a, b = mul2048_u32()
        da, db = B.to_device(a), B.to_device(b)
        r = torch.empty((a.shape[0], 128), dtype=torch.int32, device="cuda")
        n = a.shape[0]
        ms = graph_time(lambda st: check(L, L.bi_mulfull_u32(da.data_ptr(), db.data_ptr(), r.data_ptr(), 64, n, st)))
        x = torch.zeros(2, dtype=torch.int64, device="cuda")
        ms0 = graph_time(lambda st: check(L, L.bi_add_u64(x.data_ptr(), x.data_ptr(), x.data_ptr(), 1, 1, st)))
        print(json.dumps({"workload": w, "n": n, "ms": ms, "instances_per_s": n / ms * 1e3,
                          "one_limb_add_ms": ms0, "timing": "one replay of a CUDA graph of 20 launches"}))
    elif w == "batch":
        d, arena, out_limbs, nflags = B.workloads.uneven_batch(n=args.batch_n)
        din = B.to_device(arena)
        dout = torch.zeros(out_limbs, dtype=torch.int64, device="cuda")
        dfl = torch.zeros(nflags, dtype=torch.uint8, device="cuda")
        plan = B.Plan(d, len(arena), out_limbs, nflags)
        ms = event_time(stream, lambda: plan.execute(din, dout, dfl, stream=stream), args.steps, args.warmup)
        plan.close()
        print(json.dumps({"workload": w, "n": args.batch_n, "ms": ms, "instances_per_s": args.batch_n / ms * 1e3}))
    elif w == "serve":
        rates = [args.serve_rate] if args.serve_rate else None
        print(json.dumps({"workload": w, "serving": measure_serving(B, rates=rates)}))
    else:
        raise SystemExit(f"unknown workload {w}")


def summary(extra, achieved_gbs: float, peak_gbs: float):
    """The headline results of every workload in a few hundred bytes, the last
    key of the JSON line: per size the instances/s and fraction of the
    measured peak, and the ratios against the reference's own kernels."""
    if not extra:
        return None
    sm = {"addsub_sweep_frac_of_hbm_peak": round(achieved_gbs / peak_gbs, 3)}
    mu = extra.get("mul_u64_full", {})
    sm["mulfull_u64"] = {k.split("_")[0]: [v["full_instances_per_s"], v["frac_of_intpipe_peak"],
                                           v["truncated_instances_per_s"]] for k, v in mu.items()}
    sm["mulfull_u64_fields"] = "m: [full inst/s, full frac of int-pipe peak, truncated inst/s]"
    dv = extra.get("div_u64_2m_by_m", {})
    sm["div_u64_2m_by_m"] = {k.split("_")[0]: [v["instances_per_s"], v["frac_of_intpipe_peak"], v["frac_of_hbm_peak"]]
                             for k, v in dv.items()}
    sm["div_fields"] = "m: [div/s, frac of int-pipe peak in the method's own limb products, frac of HBM peak]"
    if "mul2048_u32" in extra:
        sm["c1_mulfull_u32_2048bit_inst_per_s"] = extra["mul2048_u32"]["instances_per_s"]
    sp = extra.get("mulfull_u64_small", {})
    sm["mul_u64_small"] = {k.split("_")[0]: [v["instances_per_s"], v["frac_of_intpipe_peak"],
                                             v.get("truncated_instances_per_s")] for k, v in sp.items()}
    sm["mul_u64_small_fields"] = "m: [full inst/s, full frac of int-pipe peak, truncated inst/s]"
    ub = extra.get("uneven_batch")
    if ub:
        sm["uneven_batch_100k"] = {"inst_per_s": ub["batched_inst_per_s"],
                                   "x_per_size_python": ub["speedup_vs_per_size_launch"],
                                   "x_per_size_graph": ub.get("speedup_vs_per_size_graph"),
                                   "frac_intpipe": ub.get("roofline", {}).get("frac_of_intpipe_peak"),
                                   "frac_hbm": ub.get("roofline", {}).get("frac_of_hbm_peak")}
    rk = extra.get("reference_cuda_kernels", {})
    if "add_u64_gbs" in rk:
        sm["x_vs_ref_baddKer3_add"] = {b: round(v["ours"] / v["reference_baddKer3"], 2)
                                       for b, v in rk["add_u64_gbs"].items() if v.get("reference_baddKer3")}
    if "mul_u64" in rk:
        sm["x_vs_ref_convMul5"] = {k.split("_")[0]: {
            "truncated": round(v["truncated_ours_inst_per_s"] / v["truncated_reference_inst_per_s"], 2),
            "full": (round(v["full_ours_inst_per_s"] / v["full_reference_inst_per_s"], 2)
                     if v.get("full_reference_inst_per_s") else None)} for k, v in rk["mul_u64"].items()}
    if "mul_u64_small" in rk:
        sm["x_vs_ref_convMul5_small"] = {k.split("_")[0]: {
            "truncated": round(v["truncated_ours_inst_per_s"] / v["truncated_reference_inst_per_s"], 2),
            "full": round(v["full_ours_inst_per_s"] / v["full_reference_inst_per_s"], 2)}
            for k, v in rk["mul_u64_small"].items()}
    if rk.get("mul2048_u32_full_reference_inst_per_s") and "mul2048_u32" in extra:
        sm["x_vs_ref_convMul5_c1"] = round(extra["mul2048_u32"]["instances_per_s"]
                                           / rk["mul2048_u32_full_reference_inst_per_s"], 2)
    sv = extra.get("serving", {}).get("rates_rps", {})
    sm["serve"] = {r: {"loop_p50_p99_us": [v["loop"]["p50_us"], v["loop"]["p99_us"]],
                       "launch_p99_us": v["per_request_launch"]["p99_us"],
                       "achieved_rps": v["loop"]["achieved_rps"]} for r, v in sv.items()}
    return sm


def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    import bigint_gb300 as B
    from bigint_gb300.workloads import addsub_u64_device

    B.build()
    L = B.lib()
    stream = torch.cuda.current_stream()
    sp = int(stream.cuda_stream)
    total = 1 << args.total_limbs_log2
    bits_list = [args.bits] if args.bits else BITS

    inputs = {(bits, op): addsub_u64_device(bits, seed=SEED_ADDSUB, total_limbs=total, op=op)
              for bits in bits_list for op in ("add", "sub")}
    out = torch.empty(total, dtype=torch.int64, device="cuda")
    sign = torch.empty(total // 16, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    def launch(bits, op):
        a, b = inputs[(bits, op)]
        n, m = a.shape
        if op == "add":
            check(L, L.bi_add_u64(a.data_ptr(), b.data_ptr(), out.data_ptr(), m, n, sp))
        else:
            check(L, L.bi_sub_u64(a.data_ptr(), b.data_ptr(), out.data_ptr(), sign.data_ptr(), m, n, sp))

    per_step = 0
    for (bits, op), (a, b) in inputs.items():
        per_step += 3 * a.numel() * 8 + (a.shape[0] if op == "sub" else 0)

    warm = max(3, args.warmup)
    for _ in range(warm):
        for key in inputs:
            launch(*key)
    torch.cuda.synchronize()

    events = []
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler() as clk:
        start.record(stream)
        for _ in range(args.steps):
            for key in inputs:
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                launch(*key)
                e1.record(stream)
                events.append((key, e0, e1))
        stop.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    elapsed_ms, value = whole_job(start.elapsed_time(stop), per_step, args.steps, world, device="cuda")

    per_launch = {}
    for (bits, op), e0, e1 in events:
        per_launch.setdefault(f"{op}_{bits}", []).append(e0.elapsed_time(e1))
    launch_ms = [x for v in per_launch.values() for x in v]
    avg_launch_ms = float(np.mean(launch_ms))
    bytes_per_launch = per_step / len(inputs)
    achieved = bytes_per_launch / (avg_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peaks()

    # ---- e2e through the host C-ABI entry points, and the CPU baseline on the same host buffers
    e2e_ms = 0.0
    h2d = d2h = 0
    cpu_s = 0.0
    cpu_bytes = 0
    nthreads = os.cpu_count() or 1
    ha = torch.empty(total, dtype=torch.int64, pin_memory=True)
    hb = torch.empty(total, dtype=torch.int64, pin_memory=True)
    hr = torch.empty(total, dtype=torch.int64, pin_memory=True)
    hs = torch.empty(total // 16, dtype=torch.uint8, pin_memory=True)
    e2e_steps = 0 if args.no_e2e else 1
    cpu_reps = 0 if (args.no_cpu or rank != 0) else 2
    for rep in range(max(e2e_steps, cpu_reps)):
        for (bits, op), (a, b) in inputs.items():
            n, m = a.shape
            ha[: n * m].copy_(a.view(-1))
            hb[: n * m].copy_(b.view(-1))
            torch.cuda.synchronize()
            if rep < e2e_steps:
                t0 = time.perf_counter()
                if op == "add":
                    check(L, L.bi_host_add_u64(ha.data_ptr(), hb.data_ptr(), hr.data_ptr(), m, n))
                    d2h += n * m * 8
                else:
                    check(L, L.bi_host_sub_u64(ha.data_ptr(), hb.data_ptr(), hr.data_ptr(), hs.data_ptr(), m, n))
                    d2h += n * m * 8 + n
                e2e_ms += (time.perf_counter() - t0) * 1e3
                h2d += 2 * n * m * 8
            if rep < cpu_reps:
                an = ha[: n * m].numpy().view(np.uint64).reshape(n, m)
                bn = hb[: n * m].numpy().view(np.uint64).reshape(n, m)
                cpu_s += cpu_addsub(op, an, bn, nthreads)
                cpu_bytes += 3 * n * m * 8 + (n if op == "sub" else 0)
    e2e = None
    if e2e_steps:
        e2e_t = torch.tensor([e2e_ms], device="cuda")
        if world > 1:
            dist.all_reduce(e2e_t, op=dist.ReduceOp.MAX)
        e2e = {"value": round(per_step * e2e_steps * world / (float(e2e_t.item()) / 1e3) / 1e9, 2), "unit": "GB/s",
               "h2d_bytes_per_step": h2d // e2e_steps, "d2h_bytes_per_step": d2h // e2e_steps,
               "path": "bi_host_add_u64 / bi_host_sub_u64 from pinned host buffers (the kernels read and write "
                       "them in place over the CPU-GPU link)"}
        # the link's own ceiling for this traffic: copy-engine bandwidth each way on the same pinned buffers
        dev = torch.empty(total, dtype=torch.int64, device="cuda")
        def copy_gbs(dst, src):
            for _ in range(2):
                dst.copy_(src, non_blocking=True)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(3):
                dst.copy_(src, non_blocking=True)
            e1.record()
            torch.cuda.synchronize()
            return 3 * total * 8 / (e0.elapsed_time(e1) / 1e3) / 1e9
        h2d_gbs, d2h_gbs = copy_gbs(dev, ha), copy_gbs(hr, dev)
        del dev
        t_min = max(h2d / e2e_steps / (h2d_gbs * 1e9), d2h / e2e_steps / (d2h_gbs * 1e9))
        e2e["link"] = {"h2d_gbs": round(h2d_gbs, 1), "d2h_gbs": round(d2h_gbs, 1),
                       "ceiling_gbs": round(per_step / t_min / 1e9, 1),
                       "frac": round(e2e["value"] / (per_step / t_min / 1e9), 3),
                       "note": "ceiling = the step's algorithmic bytes / the longer of its host-to-device and "
                               "device-to-host bytes at the measured copy bandwidths (both directions overlapped)"}

    extra = None
    if not args.no_extras:
        extra = measure_extra(B, L, stream, args)

    if rank == 0:
        line = {
            "metric": "add/sub sweep GB/s (u64, 2^10..2^18 bits, 2^27 limbs per operand)",
            "value": round(value, 2),
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": warm,
            "ms_per_step": round(elapsed_ms / args.steps, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": round(value / PUBLISHED_ADD_U64_GBS, 2),
            "vs_baseline_ref": "u64 add C-V3 mean 165 GB/s, GTX 1650 SUPER (thesis performance.tex:181-198)",
            "dtype": "u64",
            "data": "synthetic (splitmix64 seed 1001; 20% carry-chain instances)",
            "config": {"workload": "addsub_u64 sweep: 9 sizes 2^10..2^18 bits x {add, sub}, n = 2^27/m instances per size",
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (1 GiB per operand), no flush"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4),
                         "peak_source": "of measured (MEASURED_PEAKS.json hbm_gbs)" if peak_kind == "measured"
                         else "of fallback 6.8 TB/s",
                         "peak_note": "the denominator is a device-to-device copy (one byte read per byte written); "
                                      "add/sub reads two bytes per byte written, so a streaming kernel can read a "
                                      "little above 1.0 of it",
                         "kernel": "addsub_chunk_kernel (add and sub launches)", "bytes_per_launch": int(bytes_per_launch),
                         "avg_launch_ms": round(avg_launch_ms, 5),
                         "traffic": (ncu_traffic("addsub_chunk_kernel") or {}).get("bytes_per_launch"),
                         "traffic_source": (ncu_traffic("addsub_chunk_kernel") or {}).get("source")},
            "per_size_gbs": {k: round(3 * total * 8 / (float(np.mean(v)) / 1e3) / 1e9, 1) for k, v in per_launch.items()},
            "e2e": e2e,
            "gpu_launches": len(events),
            "clocks": clk.summary(),
            "cpu_baseline": None if not cpu_reps else {
                "value": round(cpu_bytes / cpu_s / 1e9, 3), "unit": "GB/s", "cores": nthreads, "kind": "port",
                "sample": f"the full sweep (same inputs, 2^27 limbs per size) run {cpu_reps}x: {cpu_s:.2f} s wall "
                          f"on {nthreads} threads; oracle port of ker-add.cu.h / sub.fut"},
            "extra": extra,
            "summary": summary(extra, achieved, peak),
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="addsub",
                    choices=["addsub", "add", "sub", "mul", "mul2048", "div", "divsweep", "batch", "serve"])
    ap.add_argument("--bits", type=int, default=0, help="restrict the add/sub sweep to one size")
    ap.add_argument("--total-limbs-log2", type=int, default=27)
    ap.add_argument("--mul-m", type=int, default=1024)
    ap.add_argument("--div-m", type=int, default=256)
    ap.add_argument("--div-method", default="auto", choices=["auto", "shinv", "long"])
    ap.add_argument("--batch-n", type=int, default=100_000)
    ap.add_argument("--serve-rate", type=int, default=0, help="serve workload: one offered load (requests/s)")
    ap.add_argument("--no-extras", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload != "addsub":
        run_single(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

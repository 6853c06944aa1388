#!/usr/bin/env python3
"""Benchmark of the GB300 batched big-integer library.

Headline workload (one "step"): the batched add + signed-sub sweep over u64
limbs at 2^10 .. 2^18 bits, each size filling 2^27 limbs per operand (1 GiB),
80 % uniform and 20 % carry-chain instances -- 9 sizes x {add, sub} = 18
kernel launches per step.  The metric is the reference's add bandwidth,
GB/s = 3 * n * m * 8 / t (thesis/sections/performance.tex:75-78), summed over
the step.  Operands are 1 GiB each, far larger than the 129 MB L2, so no L2
flush is needed between launches.

  * value      -- device-resident inputs, whole-job GB/s over all ranks;
  * e2e        -- the same sweep through the host C-ABI entry points
                  (bi_host_add_u64 / bi_host_sub_u64) from pinned host memory,
                  copies in and out inside the timed region;
  * roofline   -- the add/sub kernel's algorithmic bytes per launch over its
                  CUDA-event launch time, against the measured HBM copy peak;
  * cpu_baseline -- the CPU oracle port on the host cores, on a 1/8 sample.

`--impl reference` times the reference's CPU implementation of the path on
the host cores -- here the oracle port of it, all threads -- on the same
metric and workload, and prints the same JSON line with "impl": "reference".

Multi-GPU: instances are independent, so N ranks run N replicas of the step
(weak scaling, no collective on the data path; NCCL is used only for the
barrier and the max over ranks of the elapsed time).
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(REPO, "big-int_gb300"))

TOTAL_LIMBS = 1 << 27
SEED = 1001                       # workload index 1 -> seed 1000 + 1
BITS = [1 << k for k in range(10, 19)]
PUBLISHED_ADD_U64_GBS = 165.0     # mean of C-V3 u64 add over 2^10..2^18 bits, GTX 1650 SUPER
FALLBACK_HBM_GBS = 6800.0


def step_bytes(total_limbs: int = TOTAL_LIMBS) -> tuple[int, int]:
    """Algorithmic bytes of one step: (add+sub limb traffic, sign bytes)."""
    per_op = 3 * total_limbs * 8
    signs = sum(total_limbs // (b // 64) for b in BITS)
    return 2 * len(BITS) * per_op + signs, signs


def measured_peak():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic():
    """Per-launch DRAM bytes of the add/sub kernel from the committed ncu summary."""
    path = os.path.join(REPO, "profiles", "addsub_traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "100"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# CPU legs (oracle port; the library never touches these)
# ---------------------------------------------------------------------------

def cpu_sweep(nthreads: int, total_limbs: int) -> dict:
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    from bigint_gb300.workloads import addsub_u64

    O.build()
    elapsed = 0.0
    nbytes = 0
    for bits in BITS:
        for op in ("add", "sub"):
            a, b = addsub_u64(bits, seed=SEED, total_limbs=total_limbs, op=op)
            t0 = time.perf_counter()
            if op == "add":
                O.add(a, b, nthreads=nthreads)
            else:
                O.sub(a, b, nthreads=nthreads)
            elapsed += time.perf_counter() - t0
            nbytes += 3 * a.size * 8 + (a.shape[0] if op == "sub" else 0)
    return {"gbs": nbytes / elapsed / 1e9, "seconds": elapsed, "bytes": nbytes}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    sample = TOTAL_LIMBS // 8
    for _ in range(args.warmup):
        pass  # the CPU port has no warm-up state; the first timed sweep includes page faults
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        vals.append(cpu_sweep(cores, sample)["gbs"])
    wall = time.perf_counter() - t0
    v = float(np.median(vals))
    line = {
        "impl": "reference",
        "metric": "add/sub sweep GB/s (u64, 2^10..2^18 bits, 2^27 limbs per operand)",
        "value": round(v, 3), "unit": "GB/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(1000 * wall / max(1, args.steps), 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (splitmix64 seed 1001)",
        "config": {"workload": "addsub_u64 sweep 2^10..2^18 bits", "sample": "1/8 of the 2^27 limbs per size",
                   "l2": "inputs larger than L2"},
        "cpu_baseline": {"value": round(v, 3), "unit": "GB/s", "cores": cores, "kind": "port",
                         "sample": "each step: the full 9-size add+sub sweep at 2^24 limbs per operand "
                                   "(1/8 of the GPU workload); oracle port of ker-add.cu.h / sub.fut, "
                                   "one pthread per core"},
        "e2e": {"value": round(v, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# GPU leg
# ---------------------------------------------------------------------------

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

    # ---- device-resident inputs for every size and op
    inputs = {}
    for bits in BITS:
        for op in ("add", "sub"):
            inputs[(bits, op)] = addsub_u64_device(bits, seed=SEED, total_limbs=TOTAL_LIMBS, op=op)
    out = torch.empty(TOTAL_LIMBS, dtype=torch.int64, device="cuda")
    sign = torch.empty(TOTAL_LIMBS // 16, dtype=torch.uint8, device="cuda")
    torch.cuda.synchronize()

    def launch(bits, op):
        a, b = inputs[(bits, op)]
        n, m = a.shape
        if op == "add":
            st = L.bi_add_u64(a.data_ptr(), b.data_ptr(), out.data_ptr(), m, n, sp)
        else:
            st = L.bi_sub_u64(a.data_ptr(), b.data_ptr(), out.data_ptr(), sign.data_ptr(), m, n, sp)
        if st != 0:
            raise RuntimeError(f"launch failed: {L.bi_last_error().decode()}")

    def one_step(events=None):
        for bits in BITS:
            for op in ("add", "sub"):
                if events is not None:
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    launch(bits, op)
                    e1.record(stream)
                    events.append((bits, op, e0, e1))
                else:
                    launch(bits, op)

    for _ in range(max(3, args.warmup)):
        one_step()
    torch.cuda.synchronize()

    # ---- timed region (device-resident)
    events = []
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        start.record(stream)
        for _ in range(args.steps):
            one_step(events)
        stop.record(stream)
        torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    elapsed_ms = start.elapsed_time(stop)
    t = torch.tensor([elapsed_ms], device="cuda")
    if world > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    elapsed_ms = float(t.item())
    launches = len(events)

    per_step, signs = step_bytes()
    total_bytes = per_step * args.steps * world
    value = total_bytes / (elapsed_ms / 1e3) / 1e9

    kern_ms = [e0.elapsed_time(e1) for (_, _, e0, e1) in events]
    per_launch = {}
    for (bits, op, e0, e1), ms in zip(events, kern_ms):
        per_launch.setdefault(f"{op}_{bits}", []).append(ms)
    avg_launch_ms = float(np.mean(kern_ms))
    bytes_per_launch = per_step / (2 * len(BITS))
    achieved = bytes_per_launch / (avg_launch_ms / 1e3) / 1e9
    peak, peak_kind = measured_peak()
    traffic = ncu_traffic()

    # ---- e2e through the host C-ABI entry points (pinned host memory)
    e2e_ms = 0.0
    h2d = d2h = 0
    hr =torch.empty(TOTAL_LIMBS, dtype=torch.int64, pin_memory=True)
    hs = torch.empty(TOTAL_LIMBS // 16, dtype=torch.uint8, pin_memory=True)
    ha = torch.empty(TOTAL_LIMBS, dtype=torch.int64, pin_memory=True)
    hb = torch.empty(TOTAL_LIMBS, dtype=torch.int64, pin_memory=True)
    e2e_steps = max(1, min(args.steps, 2))
    for _ in range(e2e_steps):
        for bits in BITS:
            for op in ("add", "sub"):
                a, b = inputs[(bits, op)]
                n, m = a.shape
                ha.copy_(a.view(-1))
                hb.copy_(b.view(-1))
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                if op == "add":
                    st = L.bi_host_add_u64(ha.data_ptr(), hb.data_ptr(), hr.data_ptr(), m, n)
                    d2h += n * m * 8
                else:
                    st = L.bi_host_sub_u64(ha.data_ptr(), hb.data_ptr(), hr.data_ptr(), hs.data_ptr(), m, n)
                    d2h += n * m * 8 + n
                e2e_ms += (time.perf_counter() - t0) * 1e3
                h2d += 2 * n * m * 8
                if st != 0:
                    raise RuntimeError(L.bi_last_error().decode())
    e2e_t = torch.tensor([e2e_ms], device="cuda")
    if world > 1:
        dist.all_reduce(e2e_t, op=dist.ReduceOp.MAX)
    e2e_value = per_step * e2e_steps * world / (float(e2e_t.item()) / 1e3) / 1e9

    cpu = None
    if rank == 0:
        nthreads = os.cpu_count() or 1
        r = cpu_sweep(nthreads, TOTAL_LIMBS // 8)
        cpu = {"value": round(r["gbs"], 3), "unit": "GB/s", "cores": nthreads, "kind": "port",
               "sample": "the 9-size add+sub sweep at 2^24 limbs per operand (1/8 of the workload), "
                         f"{r['seconds']:.2f} s of CPU time; oracle port, one pthread per core"}

    if rank == 0:
        line = {
            "metric": "add/sub sweep GB/s (u64, 2^10..2^18 bits, 2^27 limbs per operand)",
            "value": round(value, 2),
            "unit": "GB/s",
            "n_gpus": world,
            "steps": args.steps,
            "warmup": max(3, args.warmup),
            "ms_per_step": round(elapsed_ms / args.steps, 4),
            "higher_is_better": True,
            "scaling": "weak",
            "vs_baseline": round(value / PUBLISHED_ADD_U64_GBS, 2),
            "dtype": "u64",
            "data": "synthetic (splitmix64 seed 1001; 20% carry-chain instances)",
            "config": {"workload": "addsub_u64 sweep: 9 sizes 2^10..2^18 bits x {add, sub}, "
                                   "n = 2^27/m instances per size",
                       "parallelism": f"replicas x{world}",
                       "l2": "inputs larger than L2 (1 GiB per operand), no flush"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)"
                         if peak_kind == "measured" else "fallback 6.8 TB/s",
                         "kernel": "addsub_kernel", "bytes_per_launch": int(bytes_per_launch),
                         "avg_launch_ms": round(avg_launch_ms, 5),
                         "traffic": (traffic or {}).get("bytes_per_launch")},
            "per_size_gbs": {k: round(3 * TOTAL_LIMBS * 8 / (np.mean(v) / 1e3) / 1e9, 1)
                             for k, v in per_launch.items()},
            "e2e": {"value": round(e2e_value, 2), "unit": "GB/s",
                    "h2d_bytes_per_step": h2d // e2e_steps, "d2h_bytes_per_step": d2h // e2e_steps,
                    "path": "bi_host_add_u64 / bi_host_sub_u64 from pinned host buffers"},
            "gpu_launches": launches,
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

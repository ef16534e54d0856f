"""GEMM-family throughput on GB300: split-BF16 tcgen05 vs plain FP32 SIMT.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

One step = one C = alpha*A*B + beta*C over N x N FP32 matrices (polybench gemm
initialisation, alpha=32412, beta=2123, N=8192 by default), all operands
resident in HBM.  Prints one JSON line (rank 0).  Under torchrun every rank
runs an independent replica on its own GPU (the contraction has no exchange
step), so scaling is weak and `value` sums all ranks' work over the slowest
rank's time.

`--impl reference` times the reference's CPU implementation of the same
kernel body (gemm.cpp:82-91) on the host cores, through the oracle's port of
it, on a bounded sample of the same workload.
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
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "sycl-bench_gb300"))

import numpy as np  # noqa: E402

ALPHA, BETA = 32412.0, 2123.0
PEAKS_FILE = ROOT / "MEASURED_PEAKS.json"
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}
L2_BYTES = 126 << 20  # GB300's L2 (both dies)
# DRAM bytes (read + write) per launch of the dominant kernel, keyed by
# (kernel, N, tile configuration): ncu's dram__bytes_read.sum +
# dram__bytes_write.sum from one capture of the same kernel, configuration
# and workload.
TRAFFIC_PER_LAUNCH: dict[tuple[str, int, int], float] = {
    ("bf16x3_gemm", 4096, 1): 397.3e6, ("bf16x3_gemm", 8192, 1): 2.797e9,
    ("bf16x3_gemm", 4096, 3): 462.6e6, ("bf16x3_gemm", 8192, 3): 3.163e9}


# ------------------------------------------------------------------ helpers
def polybench_gemm_init(n: int):
    """gemm.cpp:18-40 in float32 arithmetic: A=i*k/N, B=(k*j+1)/N, C=(i*j+2)/N."""
    i = np.arange(n, dtype=np.float32)[:, None]
    j = np.arange(n, dtype=np.float32)[None, :]
    nf = np.float32(n)
    ij = i * j
    return ij / nf, (ij + np.float32(1)) / nf, (ij + np.float32(2)) / nf


def load_peaks() -> tuple[dict, str]:
    if PEAKS_FILE.exists():
        try:
            return json.loads(PEAKS_FILE.read_text()), "measured"
        except (OSError, ValueError):
            pass
    return dict(FALLBACK_PEAKS), "fallback"


class NvmlSampler:
    """SM clock, its maximum, power and clock-event reasons read through NVML
    (the driver's libnvidia-ml, read-only queries) every 5 ms in a thread, so
    that a timed region of a few tens of milliseconds still holds samples.
    The device is found by its PCI bus id, as the CUDA runtime reports it."""

    # nvmlClocksEventReason bits
    REASONS = {0x8: "hw_slowdown", 0x40: "hw_thermal_slowdown", 0x20: "sw_thermal_slowdown", 0x4: "sw_power_cap"}

    def __init__(self, device: int, period_s: float = 0.005):
        import ctypes as ct
        self.ct = ct
        self.period = period_s
        self.samples: list[tuple[float, float, float, int, float]] = []
        self.stop_flag = threading.Event()
        self.thread = None
        self.nvml = ct.CDLL("libnvidia-ml.so.1")
        if self.nvml.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        rt = ct.CDLL("libcudart.so.13")
        bus = ct.create_string_buffer(64)
        if rt.cudaDeviceGetPCIBusId(bus, 64, device) != 0:
            raise OSError("cudaDeviceGetPCIBusId failed")
        self.handle = ct.c_void_p()
        if self.nvml.nvmlDeviceGetHandleByPciBusId_v2(bus, ct.byref(self.handle)) != 0:
            raise OSError("nvmlDeviceGetHandleByPciBusId failed")
        self.reasons_fn = getattr(self.nvml, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            self.nvml.nvmlDeviceGetCurrentClocksThrottleReasons

    def _one(self):
        ct = self.ct
        sm, smax, mw, rs = ct.c_uint(), ct.c_uint(), ct.c_uint(), ct.c_ulonglong()
        ok = self.nvml.nvmlDeviceGetClockInfo(self.handle, 1, ct.byref(sm)) == 0  # NVML_CLOCK_SM
        self.nvml.nvmlDeviceGetMaxClockInfo(self.handle, 1, ct.byref(smax))
        self.nvml.nvmlDeviceGetPowerUsage(self.handle, ct.byref(mw))
        self.reasons_fn(self.handle, ct.byref(rs))
        if ok:
            self.samples.append((time.time(), float(sm.value), float(smax.value), int(rs.value), mw.value / 1e3))

    def _run(self):
        while not self.stop_flag.is_set():
            self._one()
            time.sleep(self.period)

    def start(self) -> None:
        self.thread = threading.Thread(target=self._run, daemon=True)
        self.thread.start()

    def stop(self) -> None:
        self.stop_flag.set()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0: float, t1: float) -> dict:
        rows = [s for s in self.samples if t0 <= s[0] <= t1]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no NVML sample in the timed region"],
                    "samples": 0}
        reasons = sorted({name for r in rows for bit, name in self.REASONS.items() if r[3] & bit})
        return {"sm_mhz": statistics.median(r[1] for r in rows), "sm_max_mhz": max(r[2] for r in rows),
                "sm_mhz_min": min(r[1] for r in rows), "reasons": reasons, "samples": len(rows),
                "window": f"timed region ({t1 - t0:.3f} s), NVML every {self.period * 1e3:.0f} ms",
                "power_w_max": max(r[4] for r in rows)}


def clock_sampler(device: int):
    """NVML sampler when the driver library answers, else nvidia-smi every 200 ms."""
    try:
        return NvmlSampler(device)
    except (OSError, AttributeError):
        return ClockSampler(device)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms in a thread."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,utilization.gpu,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.samples: list[tuple[float, list[str]]] = []
        self.proc = None
        self.thread = None

    def start(self) -> None:
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200",
                 "-i", str(self.device)], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self) -> None:
        for line in self.proc.stdout:
            self.samples.append((time.time(), [x.strip() for x in line.split(",")]))

    def stop(self) -> None:
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        if self.thread:
            self.thread.join(timeout=5)

    def summary(self, t0: float, t1: float) -> dict:
        window = "timed"
        rows = [s for t, s in self.samples if t0 <= t <= t1]
        if len(rows) < 3:  # timed region shorter than a few sampling periods: widen to the loaded phase
            rows = [s for _, s in self.samples if len(s) > 4 and s[4].isdigit() and int(s[4]) > 0]
            window = "loaded phase (timed region shorter than the sampling period)"
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}

        def num(x):
            try:
                return float(x)
            except ValueError:
                return None
        sm = [v for v in (num(r[1]) for r in rows) if v is not None]
        smax = [v for v in (num(r[2]) for r in rows) if v is not None]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if len(r) > 6 + k and r[6 + k] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows), "window": window,
                "power_w_max": max((num(r[3]) or 0.0) for r in rows)}


class Dist:
    """torchrun rendezvous for replicas: barrier and max-over-ranks only."""

    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as td
            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local_rank)
            td.init_process_group(backend=backend)
            self.td, self.torch, self.backend = td, torch, backend

    def barrier(self) -> None:
        if self.world > 1:
            self.td.barrier()

    def max(self, x: float) -> float:
        if self.world == 1:
            return x
        dev = f"cuda:{self.local_rank}" if self.backend == "nccl" else "cpu"
        t = self.torch.tensor([x], dtype=self.torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.world > 1:
            self.td.destroy_process_group()


# ------------------------------------------------------------ GPU workload
def run_gpu(args, dist: Dist) -> dict | None:
    import gbpoly
    from gbpoly import Precision

    n = args.size
    nbytes = n * n * 4
    flops = 2.0 * n ** 3
    ctx = gbpoly.Context(dist.local_rank)
    props = ctx.device_props()
    A, B, C = polybench_gemm_init(n)
    dA, dB, dC, dC0 = ctx.upload(A), ctx.upload(B), ctx.upload(C), ctx.upload(C)

    # FP64 oracle on the GPU (DGEMM) for the error of each form
    dA64, dB64, dR = ctx.alloc(2 * nbytes), ctx.alloc(2 * nbytes), ctx.alloc(2 * nbytes)
    ctx.convert_f32_f64(dA, dA64, n * n)
    ctx.convert_f32_f64(dB, dB64, n * n)
    ctx.convert_f32_f64(dC0, dR, n * n)
    ctx.gemm_f64(n, n, n, ALPHA, dA64, n, dB64, n, BETA, dR, n)
    ctx.synchronize()
    ctx.free(dA64)
    ctx.free(dB64)

    def one(prec):
        ctx.gemm(prec, n, n, n, ALPHA, dA, n, dB, n, BETA, dC, n)

    def fresh_c():
        ctx.lib.gbpoly_memcpy_d2d(ctx.handle, gbpoly._ptr(dC), gbpoly._ptr(dC0), nbytes)

    forms = [Precision[f.strip().upper()] for f in args.forms.split(",")]
    headline = Precision.BF16X3 if Precision.BF16X3 in forms else forms[-1]
    tiers = {}
    sampler = clock_sampler(dist.local_rank)
    sampler.start()
    timed_window = (0.0, 0.0)
    windows = {}  # each form's timed region, for its clock record
    tuned = {}
    for prec in forms:
        if prec == Precision.FP32:
            continue
        if args.tile_config is not None:  # forced (profiling runs: no autotuner launches)
            tuned[prec] = min(args.tile_config, ctx.config_count(prec) - 1)
            ctx.config_set(prec, n, n, n, tuned[prec])
        else:  # tile configuration from the autotuner, before any timing
            tuned[prec] = ctx.autotune(prec, n, n, n, reps=3)[0]
    # error of every form on seeded uniform[-1, 1] inputs too (same shape, alpha, beta)
    rngu = np.random.default_rng(7)
    uA, uB, uC = (rngu.uniform(-1, 1, (n, n)).astype(np.float32) for _ in range(3))
    duA, duB, duC0, duC = ctx.upload(uA), ctx.upload(uB), ctx.upload(uC), ctx.upload(uC)
    del uA, uB
    dA64, dB64, dRu = ctx.alloc(2 * nbytes), ctx.alloc(2 * nbytes), ctx.alloc(2 * nbytes)
    ctx.convert_f32_f64(duA, dA64, n * n)
    ctx.convert_f32_f64(duB, dB64, n * n)
    ctx.convert_f32_f64(duC0, dRu, n * n)
    ctx.gemm_f64(n, n, n, ALPHA, dA64, n, dB64, n, BETA, dRu, n)
    ctx.synchronize()
    ctx.free(dA64)
    ctx.free(dB64)
    uniform_err = {}
    for prec in forms:
        ctx.lib.gbpoly_memcpy_d2d(ctx.handle, gbpoly._ptr(duC), gbpoly._ptr(duC0), nbytes)
        ctx.gemm(prec, n, n, n, ALPHA, duA, n, duB, n, BETA, duC, n)
        ctx.synchronize()
        mr, fr, _ = ctx.error_norms(duC, n, dRu, n, n, n)
        uniform_err[prec] = {"max_rel": mr, "frob_rel": fr}
    for b in (duA, duB, duC0, duC, dRu):
        ctx.free(b)

    for prec in forms:
        fresh_c()
        one(prec)
        ctx.synchronize()
        max_rel, frob, elem = ctx.error_norms(dC, n, dR, n, n, n)
        for _ in range(args.warmup):
            fresh_c()
            one(prec)
        ctx.synchronize()
        # Every timed step starts from the initial C (a device copy between the
        # step's events, outside them), so each step computes the benchmark's own
        # output and the last one is checked against FP64 below; each step is
        # bracketed by its own event pair.
        evs = [(ctx.event(), ctx.event()) for _ in range(args.steps)]
        dist.barrier()
        ctx.synchronize()
        ctx.profile_read()  # drop records of earlier launches
        ctx.profile(True)
        t0 = time.time()
        for s0, s1 in evs:
            fresh_c()
            s0.record()
            one(prec)
            s1.record()
        ctx.synchronize()
        t1 = time.time()
        ctx.profile(False)
        kernels = ctx.profile_read()
        dist.barrier()
        ms = sum(s0.elapsed_ms(s1) for s0, s1 in evs) / args.steps
        for s0, s1 in evs:
            s0.destroy()
            s1.destroy()
        ms = dist.max(ms)
        timed_err = ctx.error_norms(dC, n, dR, n, n, n)
        if prec == headline:
            timed_window = (t0, t1)
        windows[prec.name.lower()] = (t0, t1)
        top = max(kernels.items(), key=lambda kv: kv[1][1])
        tiers[prec.name.lower()] = {
            "ms_per_step": ms, "tflops": flops / (ms * 1e-3) / 1e12 * dist.world,
            "err_vs_fp64": {"max_rel": max_rel, "frob_rel": frob, "max_elem_rel": elem},
            "err_vs_fp64_uniform_inputs": uniform_err[prec],
            "kernel_launches_per_step": sum(c for c, _ in kernels.values()) / args.steps,
            "kernels": {k: {"launches": c, "avg_ms": t / c, "share": t / sum(x[1] for x in kernels.values())}
                        for k, (c, t) in kernels.items()},
            "dominant_kernel": top[0], "dominant_avg_ms": top[1][1] / top[1][0],
            "tile_config": tuned.get(prec),
            "timed_output_err_vs_fp64": {"max_rel": timed_err[0], "frob_rel": timed_err[1]},
        }
    sampler.stop()
    clocks = sampler.summary(*timed_window)
    for name, w in windows.items():  # every form's SM clock and power in its own timed region
        c = sampler.summary(*w)
        tiers[name]["clocks"] = {k: c.get(k) for k in ("sm_mhz", "sm_mhz_min", "power_w_max", "reasons", "samples")}

    # ---- end to end through the C ABI: pinned host buffers, copies inside the timed region
    import ctypes as ct
    hbuf = []
    for arr in (A, B, C):
        p = ct.c_void_p()
        gbpoly._check(ctx.lib.gbpoly_host_alloc(ctx.handle, ct.byref(p), nbytes))
        ct.memmove(p.value, arr.ctypes.data, nbytes)
        hbuf.append(p.value)
    hA, hB, hC = hbuf[0], hbuf[1], hbuf[2]
    hOut = hC  # C is read (beta != 0) and overwritten in place, as the reference's C buffer

    def e2e_step():
        # one call with host buffers: operands over the link, C back, pipelined inside the call
        ctx.gemm_host(headline, n, n, n, ALPHA, hA, n, hB, n, BETA, hOut, n)

    for _ in range(max(1, args.warmup)):
        e2e_step()
    ctx.synchronize()
    dist.barrier()
    e0, e1 = ctx.event(), ctx.event()
    e0.record()
    t_enq = time.perf_counter()
    for _ in range(args.steps):
        e2e_step()
    enqueue_ms = (time.perf_counter() - t_enq) * 1e3 / args.steps  # host time to issue one call's copies and launches
    e1.record()
    ctx.synchronize()
    e2e_ms = dist.max(e0.elapsed_ms(e1) / args.steps)
    # the host link on this machine, measured now: plain copies between the same pinned
    # buffers and device memory, one direction at a time
    dtmp = ctx.alloc(nbytes)

    def copy_ms(h2d: bool, reps: int = 5) -> float:
        for _ in range(2):
            for hp in (hA, hB, hC):
                (ctx.lib.gbpoly_memcpy_h2d(ctx.handle, gbpoly._ptr(dtmp), ct.c_void_p(hp), nbytes) if h2d else
                 ctx.lib.gbpoly_memcpy_d2h(ctx.handle, ct.c_void_p(hp), gbpoly._ptr(dtmp), nbytes))
        ctx.synchronize()
        c0, c1 = ctx.event(), ctx.event()
        c0.record()
        for _ in range(reps):
            for hp in (hA, hB, hC):
                gbpoly._check(ctx.lib.gbpoly_memcpy_h2d(ctx.handle, gbpoly._ptr(dtmp), ct.c_void_p(hp), nbytes) if h2d
                              else ctx.lib.gbpoly_memcpy_d2h(ctx.handle, ct.c_void_p(hp), gbpoly._ptr(dtmp), nbytes))
        c1.record()
        ctx.synchronize()
        return c0.elapsed_ms(c1) / (3 * reps)
    h2d_gbs = nbytes / (copy_ms(True) * 1e-3) / 1e9
    d2h_gbs = nbytes / (copy_ms(False) * 1e-3) / 1e9

    # both directions at once, as inside the e2e call (read-back of one panel
    # beside the next panels' input copies): a second context's stream copies
    # device -> host while this one copies host -> device
    ctx2 = gbpoly.Context(dist.local_rank)
    dtmp2 = ctx2.alloc(nbytes)

    def both_s(reps: int = 3) -> float:
        ctx.synchronize()
        ctx2.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            for hin, hout in ((hA, hB), (hB, hC), (hC, hA)):
                gbpoly._check(ctx.lib.gbpoly_memcpy_h2d(ctx.handle, gbpoly._ptr(dtmp), ct.c_void_p(hin), nbytes))
                gbpoly._check(ctx2.lib.gbpoly_memcpy_d2h(ctx2.handle, ct.c_void_p(hout), gbpoly._ptr(dtmp2), nbytes))
        ctx.synchronize()
        ctx2.synchronize()
        return (time.perf_counter() - t0) / (3 * reps)
    both_s(1)
    both_gbs = 2 * nbytes / both_s() / 1e9
    ctx2.free(dtmp2)
    ctx2.close()
    ctx.free(dtmp)
    h2d_only_ms = 3 * nbytes / (h2d_gbs * 1e9) * 1e3
    link = {"h2d_gbs": h2d_gbs, "d2h_gbs": d2h_gbs, "h2d_and_d2h_at_once_total_gbs": both_gbs,
            "host_enqueue_ms_per_call": enqueue_ms,
            "h2d_bytes_alone_ms": h2d_only_ms, "e2e_frac_of_h2d_bound": h2d_only_ms / e2e_ms,
            "measured": "plain pinned cudaMemcpyAsync of N^2 x 4 B, same buffers, same run: one direction at a time, "
                        "then both at once on two streams (host clock)"}
    for p in (hA, hB, hC):
        ctx.lib.gbpoly_host_free(ctx.handle, ct.c_void_p(p))

    grouped = None if args.no_grouped else run_grouped_workload(ctx, args)
    family = None if args.no_family else run_family(ctx, args)
    neighbours = None if args.no_neighbours else run_neighbours(ctx, args)
    small_k = None if args.no_small_k else run_small_k(ctx, args)

    head = tiers[headline.name.lower()]
    peaks, peak_kind = load_peaks()
    kernel_tflops = flops / (head["dominant_avg_ms"] * 1e-3) / 1e12
    if headline == Precision.FP32:
        # FFMA pipe: SMs x 128 lanes x 2 FLOP x max SM clock (no measured FP32 figure exists)
        clk_mhz = clocks.get("sm_max_mhz") or peaks.get("sm_max_mhz") or props["sm_clock_khz"] / 1e3
        peak = props["sm_count"] * 128 * 2 * clk_mhz * 1e6 / 1e12
        roof = {"bound": "fp32_simt", "achieved": kernel_tflops, "peak": peak, "unit": "TFLOP/s",
                "frac": kernel_tflops / peak, "traffic": None,
                "peak_source": f"computed: {props['sm_count']} SMs x 128 FFMA lanes x 2 x {clk_mhz:.0f} MHz"}
    else:
        # BF16-MMA equivalents per algorithmic multiply-add (a TF32 MMA runs at half the BF16 rate):
        # bf16x3 and fp16x3 3, tf32x3 and bf16x6 6, tf32 2.  The form's ceiling is the BF16 peak divided by that.
        mma_per_mac = {Precision.BF16X3: 3, Precision.FP16X3: 3, Precision.TF32X3: 6, Precision.BF16X6: 6,
                       Precision.TF32: 2,
                       Precision.FP8: 0.5}[headline]
        bf16 = peaks["bf16_tflops"]
        peak = bf16 / mma_per_mac
        roof = {"bound": "tensor", "achieved": kernel_tflops, "peak": peak, "unit": "TFLOP/s",
                "frac": kernel_tflops / peak, "traffic": TRAFFIC_PER_LAUNCH.get((head["dominant_kernel"], n, head["tile_config"])),
                "kernel": head["dominant_kernel"], "kernel_avg_ms": head["dominant_avg_ms"],
                "peak_source": f"{bf16} TFLOP/s dense BF16 burst ({peak_kind}) / {mma_per_mac} BF16 MMAs per "
                               f"multiply-add",
                "frac_of_bf16_peak_tensor_work": mma_per_mac * kernel_tflops / bf16}
    ctx.close()
    return {
        "value": head["tflops"], "ms_per_step": head["ms_per_step"], "tiers": tiers, "clocks": clocks,
        "roofline": roof, "headline": headline.name.lower(),
        "e2e": {"value": flops / (e2e_ms * 1e-3) / 1e12 * dist.world, "unit": "TFLOP/s",
                "h2d_bytes_per_step": 3 * nbytes, "d2h_bytes_per_step": nbytes, "ms_per_step": e2e_ms,
                "link": link},
        "err_vs_fp64": {"form": headline.name.lower(), "polybench_inputs": head["err_vs_fp64"],
                        "uniform_inputs": head["err_vs_fp64_uniform_inputs"],
                        "timed_output": head["timed_output_err_vs_fp64"]},
        "matched_error": matched_error(tiers),
        "gpu_launches": int(round(args.steps * head["kernel_launches_per_step"])),
        "device": props, "peak_kind": peak_kind, "grouped": grouped, "family": family,
        "neighbours": neighbours, "small_k": small_k,
    }


# the arithmetic each form computes in (inputs and outputs are FP32 for every form)
DTYPE_OF_FORM = {
    "fp32": "f32",
    "bf16x3": "bf16x3 (f32 in/out, bf16 hi/lo products, f32 accumulate)",
    "bf16x6": "bf16x6 (f32 in/out, three bf16 terms, 6 products, f32 accumulate)",
    "fp16x3": "fp16x3 (f32 in/out, fp16 hi/lo of power-of-two-scaled 64x64 blocks, f32 accumulate)",
    "tf32x3": "tf32x3 (f32 in/out, tf32 hi/lo products, f32 accumulate)",
    "tf32": "tf32 (f32 in/out, f32 accumulate)",
    "fp8": "e4m3 (f32 in/out, one scale per 128x128 block, f32 accumulate)",
}


def matched_error(tiers: dict) -> dict | None:
    """The fastest tensor-core form whose normwise and Frobenius errors against
    FP64 are both no larger than plain FP32's, on the polybench and on the
    uniform[-1, 1] inputs, with its throughput over FP32's."""
    f32 = tiers.get("fp32")
    if not f32:
        return None

    def within(t):
        return all(t[key][m] <= f32[key][m] for key in ("err_vs_fp64", "err_vs_fp64_uniform_inputs")
                   for m in ("max_rel", "frob_rel"))
    ok = {name: t for name, t in tiers.items() if name != "fp32" and within(t)}
    out = {"criterion": "max-normwise and Frobenius error vs FP64 <= plain FP32's, polybench and uniform[-1,1] "
                        "inputs, same N",
           "forms_meeting_it": sorted(ok), "fp32_tflops": f32["tflops"]}
    if ok:
        best = max(ok, key=lambda k: ok[k]["tflops"])
        out.update(form=best, tflops=ok[best]["tflops"], vs_fp32=ok[best]["tflops"] / f32["tflops"])
    return out


def run_family(ctx, args) -> dict:
    """The rest of the GEMM family at N = args.family_size, polybench inputs (and,
    for the errors only, seeded normal(0, 1) inputs through the same chains):
    2mm (C += A.B; E = C.D) and 3mm (E = A.B; F = C.D; G = E.F) with the stages
    of the tensor-core forms captured in one CUDA graph, syrk (C = a A.A^T + b C)
    and syr2k (C = a (A.B^T + B.A^T) + b C) with a = 32412, b = 2123 (rates in
    unique-output FLOPs), and the FP64 forms of syrk/syr2k timed alongside.  Errors against an FP64 chain
    computed on the GPU: every stage of 2mm/3mm, and the final output."""
    import gbpoly
    from gbpoly import Precision

    n = args.family_size
    nb = n * n * 4
    i = np.arange(n, dtype=np.float32)[:, None]
    j = np.arange(n, dtype=np.float32)[None, :]
    nf = np.float32(n)
    ij = i * j
    mats = {"ij": ij / nf, "ij1": (ij + np.float32(1)) / nf, "ij2": (ij + np.float32(2)) / nf,
            "i(j+1)": (i * (j + np.float32(1))) / nf, "i(j+2)": (i * (j + np.float32(2))) / nf,
            "i(j+3)": (i * (j + np.float32(3))) / nf}
    dev = {k: ctx.upload(v) for k, v in mats.items()}
    del mats
    forms = [Precision.FP32, Precision.BF16X3, Precision.BF16X6, Precision.FP16X3]
    work = [ctx.alloc(nb) for _ in range(3)]
    ref64 = [ctx.alloc(2 * nb) for _ in range(4)]
    out = {"size": n}

    def to64(src, dst):
        ctx.convert_f32_f64(src, dst, n * n)

    def dgemm(a, b, c, alpha, beta, op_b=gbpoly.Op.N):
        ctx.gemm_f64(n, n, n, alpha, a, n, b, n, beta, c, n, op_b=op_b)

    def time_steps(step, flops):
        for _ in range(args.warmup):
            step()
        ctx.synchronize()
        e0, e1 = ctx.event(), ctx.event()
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        ctx.synchronize()
        ms = e0.elapsed_ms(e1) / args.steps
        return {"ms_per_step": ms, "tflops": flops / (ms * 1e-3) / 1e12}

    def err(c32, r64):
        mr, fr, _ = ctx.error_norms(c32, n, r64, n, n, n)
        return {"max_rel": mr, "frob_rel": fr}

    def graph_of(fn):
        ctx.graph_begin()
        fn()
        return ctx.graph_end()

    # ---- 2mm: C += A.B (A = ij, B = i(j+1), C = i(j+3)), E = C.D (D = i(j+2))
    A, B, Cin, D = dev["ij"], dev["i(j+1)"], dev["i(j+3)"], dev["i(j+2)"]
    a64, b64, c64, e64 = ref64
    to64(A, a64); to64(B, b64); to64(Cin, c64)
    dgemm(a64, b64, c64, 1.0, 1.0)                 # stage 1 in FP64
    to64(D, b64)
    dgemm(c64, b64, e64, 1.0, 0.0)                 # stage 2 in FP64
    C, E = work[0], work[1]
    res = {}
    for prec in forms:
        ctx.workspace_reserve(ctx.workspace_query(prec, n, n, n))

        def stages(prec=prec):
            ctx.gemm(prec, n, n, n, 1.0, A, n, B, n, 1.0, C, n)
            ctx.gemm(prec, n, n, n, 1.0, C, n, D, n, 0.0, E, n)
        ctx.lib.gbpoly_memcpy_d2d(ctx.handle, gbpoly._ptr(C), gbpoly._ptr(Cin), nb)
        stages()
        ctx.synchronize()
        r = {"stage1_C": err(C, c64), "end_to_end_E": err(E, e64)}
        g = graph_of(stages) if prec != Precision.FP32 else None
        r.update(time_steps((lambda: ctx.graph_launch(g)) if g else stages, 4.0 * n ** 3))
        r["mode"] = "one CUDA graph" if g else "two launches"
        if g:
            ctx.graph_destroy(g)
        res[prec.name.lower()] = r
    out["2mm"] = res

    # ---- 3mm: E = A.B, F = C.D, G = E.F (A = ij, B = i(j+1), C = i(j+3), D = i(j+2))
    Cm = dev["i(j+3)"]
    to64(A, a64); to64(B, b64)
    dgemm(a64, b64, c64, 1.0, 0.0)                 # E64 in c64
    to64(Cm, a64); to64(D, b64)
    dgemm(a64, b64, e64, 1.0, 0.0)                 # F64 in e64
    g64 = ref64[0]
    dgemm(c64, e64, g64, 1.0, 0.0)                 # G64 (overwrites a64, no longer needed)
    E, F, G = work
    res = {}
    for prec in forms:
        # the split forms: E and F (independent) as one grouped launch, then G
        plan = None if prec == Precision.FP32 else ctx.grouped_plan(prec, ctx.descs([
            {"M": n, "N": n, "K": n, "alpha": 1.0, "beta": 0.0, "A": A, "lda": n, "B": B, "ldb": n, "C": E, "ldc": n},
            {"M": n, "N": n, "K": n, "alpha": 1.0, "beta": 0.0, "A": Cm, "lda": n, "B": D, "ldb": n, "C": F,
             "ldc": n}]))

        def stages(prec=prec, plan=plan):
            if plan is None:
                ctx.gemm(prec, n, n, n, 1.0, A, n, B, n, 0.0, E, n)
                ctx.gemm(prec, n, n, n, 1.0, Cm, n, D, n, 0.0, F, n)
            else:
                ctx.grouped_run(plan)
            ctx.gemm(prec, n, n, n, 1.0, E, n, F, n, 0.0, G, n)
        stages()
        ctx.synchronize()
        r = {"stage1_E": err(E, c64), "stage2_F": err(F, e64), "end_to_end_G": err(G, g64)}
        g = graph_of(stages) if prec != Precision.FP32 else None
        r.update(time_steps((lambda: ctx.graph_launch(g)) if g else stages, 6.0 * n ** 3))
        r["mode"] = "grouped E,F + G in one CUDA graph" if g else "three launches"
        if g:
            ctx.graph_destroy(g)
        if plan is not None:
            ctx.grouped_destroy(plan)
        res[prec.name.lower()] = r
    out["3mm"] = res

    # ---- syrk / syr2k, alpha = 32412, beta = 2123 (A = ij, B = ij1, C = ij2), FP64 form alongside
    al, be = 32412.0, 2123.0
    A, B, C0 = dev["ij"], dev["ij1"], dev["ij2"]
    C = work[0]
    a64, b64, r64, c64w = ref64
    to64(A, a64); to64(B, b64)
    for name in ("syrk", "syr2k"):
        to64(C0, r64)
        dgemm(a64, a64 if name == "syrk" else b64, r64, al, be, op_b=gbpoly.Op.T)
        if name == "syr2k":
            dgemm(b64, a64, r64, al, 1.0, op_b=gbpoly.Op.T)
        res = {}
        # unique-output FLOPs: n (n + 1) / 2 outputs of 2n (syrk) or 4n (syr2k) FLOPs; both forms compute
        # the lower triangle of tiles and mirror it, so the full-square count would overstate the rate
        flops = (1.0 if name == "syrk" else 2.0) * n * n * (n + 1)
        for prec in forms:
            def step(prec=prec):
                if name == "syrk":
                    ctx.syrk(prec, n, n, al, A, n, be, C, n)
                else:
                    ctx.syr2k(prec, n, n, al, A, n, B, n, be, C, n)
            ctx.lib.gbpoly_memcpy_d2d(ctx.handle, gbpoly._ptr(C), gbpoly._ptr(C0), nb)
            step()
            ctx.synchronize()
            r = {"output": err(C, r64)}
            r.update(time_steps(step, flops))
            res[prec.name.lower()] = r
        to64(C0, c64w)

        def step64():
            if name == "syrk":
                ctx.syrk_f64(n, n, al, a64, n, be, c64w, n)
            else:
                ctx.syr2k_f64(n, n, al, a64, n, b64, n, be, c64w, n)
        saved = (args.steps, args.warmup)
        args.steps, args.warmup = 2, 1  # the FP64 pipe is ~1/64 of FP32: two timed launches
        res["fp64"] = time_steps(step64, flops)
        args.steps, args.warmup = saved
        out[name] = res
    # ---- the same chains on seeded normal(0, 1) inputs (errors only; seed 4096)
    rng = np.random.default_rng(4096)
    nA, nB, nC, nD = (ctx.upload(rng.standard_normal((n, n)).astype(np.float32)) for _ in range(4))
    a64, b64, c64, e64 = ref64
    to64(nA, a64); to64(nB, b64); to64(nC, c64)
    dgemm(a64, b64, c64, 1.0, 1.0)
    to64(nD, b64)
    dgemm(c64, b64, e64, 1.0, 0.0)
    for prec in forms:
        C, E = work[0], work[1]
        ctx.lib.gbpoly_memcpy_d2d(ctx.handle, gbpoly._ptr(C), gbpoly._ptr(nC), nb)
        ctx.gemm(prec, n, n, n, 1.0, nA, n, nB, n, 1.0, C, n)
        ctx.gemm(prec, n, n, n, 1.0, C, n, nD, n, 0.0, E, n)
        ctx.synchronize()
        out["2mm"][prec.name.lower()]["normal01"] = {"stage1_C": err(C, c64), "end_to_end_E": err(E, e64)}
    to64(nA, a64); to64(nB, b64)
    dgemm(a64, b64, c64, 1.0, 0.0)                 # E64
    to64(nC, a64); to64(nD, b64)
    dgemm(a64, b64, e64, 1.0, 0.0)                 # F64
    g64 = ref64[0]
    dgemm(c64, e64, g64, 1.0, 0.0)                 # G64
    for prec in forms:
        E, F, G = work
        ctx.gemm(prec, n, n, n, 1.0, nA, n, nB, n, 0.0, E, n)
        ctx.gemm(prec, n, n, n, 1.0, nC, n, nD, n, 0.0, F, n)
        ctx.gemm(prec, n, n, n, 1.0, E, n, F, n, 0.0, G, n)
        ctx.synchronize()
        out["3mm"][prec.name.lower()]["normal01"] = {"stage1_E": err(E, c64), "stage2_F": err(F, e64),
                                                     "end_to_end_G": err(G, g64)}
    a64, b64, r64, _ = ref64
    to64(nA, a64); to64(nB, b64)
    C = work[0]
    for name in ("syrk", "syr2k"):
        to64(nC, r64)
        dgemm(a64, a64 if name == "syrk" else b64, r64, al, be, op_b=gbpoly.Op.T)
        if name == "syr2k":
            dgemm(b64, a64, r64, al, 1.0, op_b=gbpoly.Op.T)
        for prec in forms:
            ctx.lib.gbpoly_memcpy_d2d(ctx.handle, gbpoly._ptr(C), gbpoly._ptr(nC), nb)
            if name == "syrk":
                ctx.syrk(prec, n, n, al, nA, n, be, C, n)
            else:
                ctx.syr2k(prec, n, n, al, nA, n, nB, n, be, C, n)
            ctx.synchronize()
            out[name][prec.name.lower()]["normal01"] = {"output": err(C, r64)}
    for b in list(dev.values()) + work + ref64 + [nA, nB, nC, nD]:
        ctx.free(b)
    for k in ("2mm", "3mm", "syrk", "syr2k"):
        out[k]["speedup_bf16x3_vs_fp32"] = out[k]["bf16x3"]["tflops"] / out[k]["fp32"]["tflops"]
    out["normal01_inputs"] = "seeded normal(0, 1) A, B, C, D (numpy default_rng(4096)), same chains, alpha and beta"
    return out


def run_small_k(ctx, args) -> dict:
    """GEMMs whose K is too short for the tensor or FMA pipes to bound them:
    C = A.B + C at M = N = args.size, K in {32, 64, 128, 256, 512}, seeded
    uniform[-1, 1] inputs, fp32 and bf16x3.  The bound is HBM: every call
    reads and writes C (M N 8 bytes) and reads A and B ((M + N) K 4 bytes);
    reported as those algorithmic bytes per second against the measured copy
    bandwidth, with TFLOP/s and the per-kernel split (bf16x3: split pass and
    tensor-core kernel)."""
    import gbpoly
    from gbpoly import Precision

    n = args.size
    peaks, _ = load_peaks()
    hbm = peaks.get("hbm_gbs")
    rng = np.random.default_rng(64)
    dC = ctx.upload(rng.uniform(-1, 1, (n, n)).astype(np.float32))
    out = {"m_n": n, "beta": 1.0, "bytes": "M N 8 (C read and written) + (M + N) K 4 (A, B read)"}
    steps = max(args.steps, 5)
    for K in (32, 64, 128, 256, 512):
        dA = ctx.upload(rng.uniform(-1, 1, (n, K)).astype(np.float32))
        dB = ctx.upload(rng.uniform(-1, 1, (K, n)).astype(np.float32))
        row = {}
        for prec in (Precision.FP32, Precision.BF16X3):
            ctx.workspace_reserve(ctx.workspace_query(prec, n, n, K))

            def step(prec=prec):
                ctx.gemm(prec, n, n, K, 1.0, dA, K, dB, n, 1.0, dC, n)
            for _ in range(args.warmup):
                step()
            ctx.synchronize()
            e0, e1 = ctx.event(), ctx.event()
            e0.record()
            for _ in range(steps):
                step()
            e1.record()
            ctx.synchronize()
            ms = e0.elapsed_ms(e1) / steps
            ctx.profile(True)
            ctx.profile_read()
            for _ in range(steps):
                step()
            kernels = {k: round(t / c * 1e3, 2) for k, (c, t) in ctx.profile_read().items()}
            ctx.profile(False)
            gbs = (n * n * 8 + 2 * n * K * 4) / (ms * 1e-3) / 1e9
            row[prec.name.lower()] = {"us_per_call": ms * 1e3, "tflops": 2.0 * n * n * K / (ms * 1e-3) / 1e12,
                                      "gbs": gbs, "frac_of_hbm": gbs / hbm if hbm else None,
                                      "kernel_us": kernels}
        out[f"K={K}"] = row
        ctx.free(dA)
        ctx.free(dB)
    ctx.free(dC)
    return out


def run_neighbours(ctx, args) -> dict:
    """The benchmarks beside the contraction family, on their own inputs:
      * covariance and correlation at N = args.family_size: column statistics,
        centring into a packed copy and the symmetric X^T.X contraction (fp32,
        bf16x3, tf32x3), unique-output FLOPs, error against an FP64 pipeline
        (statistics in numpy FP64, contraction by DGEMM on the GPU);
      * matmulchain at N = args.family_size: R = (A.B).(C.D) on identities
        (exact result checked), fp32 as three launches, bf16x3 as one graph of
        a grouped P/Q launch and the R launch;
      * atax at N = 4096 and bicg, mvt, gesummv at N = 16384 (the suite
        runner's sizes, bin/run-suite): matrix bytes over time against the
        HBM peak, launches back to back."""
    import gbpoly
    from gbpoly import Op, Precision

    n = args.family_size
    out = {"size": n}
    peaks, _ = load_peaks()
    hbm = peaks.get("hbm_gbs")

    flush_buf = None

    def time_steps(step, steps=None, warmup=None, flush=False):
        """Mean ms per step.  flush: an operand smaller than L2 (atax at the
        suite's 4096: 64 MB) would stay in L2 across back-to-back calls, so
        each timed step gets its own event pair and a 512 MB write between
        steps, outside the events, evicts it."""
        nonlocal flush_buf
        steps, warmup = steps or args.steps, warmup or args.warmup
        for _ in range(warmup):
            step()
        ctx.synchronize()
        if flush:
            if flush_buf is None:
                flush_buf = ctx.alloc(512 << 20)
            evs = [(ctx.event(), ctx.event()) for _ in range(steps)]
            for a, b in evs:
                ctx.memset(flush_buf, 1, 512 << 20)
                a.record()
                step()
                b.record()
            ctx.synchronize()
            ms = sum(a.elapsed_ms(b) for a, b in evs) / steps
            for a, b in evs:
                a.destroy()
                b.destroy()
            return ms
        e0, e1 = ctx.event(), ctx.event()
        e0.record()
        for _ in range(steps):
            step()
        e1.record()
        ctx.synchronize()
        ms = e0.elapsed_ms(e1) / steps
        e0.destroy()
        e1.destroy()
        return ms

    # ---- covariance / correlation: (n+1) x (n+1) arrays used from index 1
    ld, ldp = n + 1, (n + 31) // 32 * 32
    i = np.arange(n + 1, dtype=np.float32)
    cov = np.zeros((ld, ld), np.float32)
    cov[:n, :n] = (i[:n, None] * i[None, :n]) / np.float32(n)             # covariance.cpp:20-29
    flat = np.zeros(ld * ld, np.float32)
    for r in range(n + 1):                                               # correlation.cpp:23-33 (row stride n)
        flat[r * n: r * n + n + 1] = (np.float32(r) * i) / np.float32(n + 1)
    corr = flat.reshape(ld, ld)
    del flat
    float_n = 3214212.01
    stats = {}
    for name, data in (("covariance", cov), ("correlation", corr)):
        x = data[1:, 1:].astype(np.float64)
        x = x - x.sum(axis=0) / float(np.float32(float_n))
        if name == "correlation":
            sd = np.sqrt((x * x).sum(axis=0) / float_n)
            sd[sd <= 0.005] = 1.0
            x = x / np.sqrt(float_n) / sd
        dX64, dR64 = ctx.upload(np.ascontiguousarray(x)), ctx.alloc(n * n * 8)
        del x
        ctx.gemm_f64(n, n, n, 1.0, dX64, n, dX64, n, 0.0, dR64, n, op_a=Op.T)
        ctx.free(dX64)
        dD, dMu, dSd = ctx.upload(data), ctx.alloc(ld * 4), ctx.alloc(ld * 4)
        dS, dY = ctx.alloc(ld * ld * 4), ctx.alloc(n * ldp * 4)
        ctx.lib.gbpoly_memset(ctx.handle, gbpoly._ptr(dS), 0, ld * ld * 4)
        X, mu, sdp, S = dD.ptr + (ld + 1) * 4, dMu.ptr + 4, dSd.ptr + 4, dS.ptr + (ld + 1) * 4
        res = {}
        for prec in (Precision.FP32, Precision.BF16X3, Precision.TF32X3):
            def step(prec=prec):
                # the drop-in's calls: fp32 centres into a packed copy and contracts it,
                # the split forms centre inside their split pass (gbpoly_covariance_f32)
                ctx.column_mean(n, n, X, ld, np.float32(float_n), mu)
                sd_arg, div = None, np.float32(1.0)
                if name == "correlation":
                    ctx.column_stddev(n, n, X, ld, mu, np.float32(float_n), np.float32(0.005), sdp)
                    sd_arg, div = sdp, np.float32(np.sqrt(float_n))
                if prec == Precision.FP32:
                    ctx.center_columns(n, n, X, ld, mu, sd_arg, div, dY, ldp)
                    ctx.gemm(prec, n, n, n, 1.0, dY, ldp, dY, ldp, 0.0, S, ld, op_a=Op.T, op_b=Op.N)
                else:
                    ctx.covariance(prec, n, n, X, ld, mu, sd_arg, div, S, ld)
                if name == "correlation":
                    ctx.set_diagonal(n, 1.0, S, ld)
            step()
            ctx.synchronize()
            got = ctx.download(dS, (ld, ld))[1:, 1:]
            ref = ctx.download(dR64, (n, n), np.float64)
            if name == "correlation":
                np.fill_diagonal(ref, 1.0)
            e = got.astype(np.float64) - ref
            ms = time_steps(step)
            flops = n * n * (n + 1) if name == "covariance" else n * n * (n - 1)
            res[prec.name.lower()] = {"ms_per_step": ms, "tflops": flops / (ms * 1e-3) / 1e12,
                                      "frob_rel": float(np.linalg.norm(e) / np.linalg.norm(ref)),
                                      "max_rel": float(np.abs(e).max() / np.abs(ref).max())}
            del got, e, ref
        res["speedup_bf16x3_vs_fp32"] = res["bf16x3"]["tflops"] / res["fp32"]["tflops"]
        stats[name] = res
        for b in (dD, dMu, dSd, dS, dY, dR64):
            ctx.free(b)
    del cov, corr
    out.update(stats)

    # ---- matmulchain on identities: P = A.B, Q = C.D, R = P.Q
    eye = np.eye(n, dtype=np.float32)
    mats = [ctx.upload(eye) for _ in range(4)]
    P, Q, R = (ctx.alloc(n * n * 4) for _ in range(3))
    res = {}
    for prec in (Precision.FP32, Precision.BF16X3):
        plan = ctx.grouped_plan(prec, ctx.descs([
            {"M": n, "N": n, "K": n, "alpha": 1.0, "beta": 0.0, "A": mats[0], "lda": n, "B": mats[1], "ldb": n,
             "C": P, "ldc": n},
            {"M": n, "N": n, "K": n, "alpha": 1.0, "beta": 0.0, "A": mats[2], "lda": n, "B": mats[3], "ldb": n,
             "C": Q, "ldc": n}]))
        ctx.workspace_reserve(ctx.workspace_query(prec, n, n, n))

        def chain(prec=prec, plan=plan):
            if prec == Precision.FP32:
                ctx.gemm(prec, n, n, n, 1.0, mats[0], n, mats[1], n, 0.0, P, n)
                ctx.gemm(prec, n, n, n, 1.0, mats[2], n, mats[3], n, 0.0, Q, n)
            else:
                ctx.grouped_run(plan)
            ctx.gemm(prec, n, n, n, 1.0, P, n, Q, n, 0.0, R, n)
        chain()
        ctx.synchronize()
        exact = bool(np.array_equal(ctx.download(R, (n, n)), eye))
        g = None
        if prec != Precision.FP32:
            ctx.graph_begin()
            chain()
            g = ctx.graph_end()
        ms = time_steps((lambda: ctx.graph_launch(g)) if g else chain)
        res[prec.name.lower()] = {"ms_per_step": ms, "tflops": 6.0 * n ** 3 / (ms * 1e-3) / 1e12,
                                  "identity_exact": exact,
                                  "mode": "grouped P,Q + R in one CUDA graph" if g else "three launches"}
        if g:
            ctx.graph_destroy(g)
        ctx.grouped_destroy(plan)
    res["speedup_bf16x3_vs_fp32"] = res["bf16x3"]["tflops"] / res["fp32"]["tflops"]
    out["matmulchain"] = res
    for b in mats + [P, Q, R]:
        ctx.free(b)
    del eye

    # ---- matrix-vector benchmarks at the suite runner's sizes
    mv = {}
    for name, m in (("atax", 4096), ("bicg", 16384), ("mvt", 16384), ("gesummv", 16384)):
        rng = np.random.default_rng(11)
        A = rng.uniform(-1, 1, (m, m)).astype(np.float32)
        v1, v2 = (rng.uniform(-1, 1, m).astype(np.float32) for _ in range(2))
        dA, d1, d2 = ctx.upload(A), ctx.upload(v1), ctx.upload(v2)
        y1, y2 = ctx.upload(np.zeros(m, np.float32)), ctx.upload(np.zeros(m, np.float32))
        dB = ctx.upload(A[::-1].copy()) if name == "gesummv" else None
        a64 = A.astype(np.float64)
        if name == "atax":
            # tmp += A x, y += A^T tmp in one call; from zero tmp and y the first call gives A^T A x
            def step():
                ctx.atax(m, m, dA, m, d1, y1, y2)
            t = a64 @ v1.astype(np.float64)
            refs, outs, passes = [a64.T @ t], [y2], 1
        elif name == "bicg":
            def step():
                ctx.gemv_pair(m, m, dA, m, [(Op.T, 1.0, 0.0, d1, y1), (Op.N, 1.0, 0.0, d2, y2)])
            refs, outs, passes = [a64.T @ v1.astype(np.float64), a64 @ v2.astype(np.float64)], [y1, y2], 1
        elif name == "mvt":
            def step():
                ctx.gemv_pair(m, m, dA, m, [(Op.N, 1.0, 0.0, d1, y1), (Op.N, 1.0, 0.0, d2, y2)])
            refs, outs, passes = [a64 @ v1.astype(np.float64), a64 @ v2.astype(np.float64)], [y1, y2], 1
        else:
            # tmp += A x; y = tmp + (y + B x): from zero tmp and y, the first call gives A x + B x
            def step():
                ctx.gesummv(m, m, 1.0, dA, m, dB, m, d1, 1.0, y1, y2)
            refs = [a64 @ v1.astype(np.float64) + a64[::-1] @ v1.astype(np.float64)]
            outs, passes = [y2], 2
        step()
        ctx.synchronize()
        errs = [float(np.linalg.norm(ctx.download(o, (m,)).astype(np.float64) - r) / np.linalg.norm(r))
                for o, r in zip(outs, refs)]
        matrix_bytes = (2 if name == "gesummv" else 1) * m * m * 4
        l2_resident = matrix_bytes < 2 * L2_BYTES
        ms = time_steps(step, steps=max(args.steps, 20), flush=l2_resident)
        gbs = matrix_bytes / (ms * 1e-3) / 1e9
        mv[name] = {"size": m, "us_per_call": ms * 1e3, "matrix_gbs": gbs,
                    "frac_of_hbm": gbs / hbm if hbm else None, "matrix_passes": passes,
                    "l2": "flushed between steps (512 MB write outside the step's events)" if l2_resident else
                          "matrix larger than L2",
                    "frob_rel_vs_fp64": max(errs)}
        for b in (dA, d1, d2, y1, y2) + ((dB,) if dB is not None else ()):
            ctx.free(b)
        del A, a64
    out["matrix_vector"] = mv
    return out


def run_grouped_workload(ctx, args) -> dict:
    """512 independent GEMMs C = A.B + 0.5 C, M, N, K log-uniform in [64, 2048]
    (seed 2024), entries uniform[-1, 1] times a per-matrix scale log-uniform in
    [1e-3, 1e3]: one grouped tensor-core plan (split pass + one persistent
    launch) replayed as a CUDA graph, against one plain FP32 launch per GEMM;
    per-matrix Frobenius error against an FP64 DGEMM on the GPU."""
    import gbpoly
    from gbpoly import Precision

    rng = np.random.default_rng(2024)
    count = args.grouped_count
    lo, hi = np.log(64), np.log(2048)
    shapes = [tuple(int(np.exp(rng.uniform(lo, hi))) for _ in range(3)) for _ in range(count)]
    items, mats = [], []
    for (M, N, K) in shapes:
        sc = float(np.exp(rng.uniform(np.log(1e-3), np.log(1e3))))
        A = (rng.uniform(-1, 1, (M, K)) * sc).astype(np.float32)
        B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
        C = rng.uniform(-1, 1, (M, N)).astype(np.float32)
        dA, dB, dC = ctx.upload(A), ctx.upload(B), ctx.upload(C)
        items.append(dict(M=M, N=N, K=K, alpha=1.0, beta=0.5, A=dA, lda=K, B=dB, ldb=N, C=dC, ldc=N))
        mats.append((C, dA, dB, dC))
    flops = float(sum(2 * M * N * K for M, N, K in shapes))

    # FP64 reference per problem (GPU DGEMM), kept on the device
    refs = []
    for (M, N, K), (C, dA, dB, dC) in zip(shapes, mats):
        a64, b64, r64 = ctx.alloc(M * K * 8), ctx.alloc(K * N * 8), ctx.alloc(M * N * 8)
        ctx.convert_f32_f64(dA, a64, M * K)
        ctx.convert_f32_f64(dB, b64, K * N)
        ctx.convert_f32_f64(dC, r64, M * N)
        ctx.gemm_f64(M, N, K, 1.0, a64, K, b64, N, 0.5, r64, N)
        ctx.free(a64)
        ctx.free(b64)
        refs.append(r64)
    ctx.synchronize()

    def reset_c():
        for C, _, _, dC in mats:
            ctx.h2d(dC, C)

    def errors():
        e = [ctx.error_norms(dC, N, r, N, M, N)[1] for (M, N, K), (_, _, _, dC), r in zip(shapes, mats, refs)]
        return {"frob_rel_max": max(e), "frob_rel_median": float(np.median(e))}

    out = {"workload": f"{count} GEMMs C=A.B+0.5C, M,N,K log-uniform [64,2048] seed 2024, per-matrix scale "
                       f"log-uniform [1e-3,1e3]", "flops_per_step": flops}
    descs = ctx.descs(items)
    for prec, mode in ((Precision.FP32, "per-GEMM launches"), (Precision.BF16X3, "grouped plan in a CUDA graph"),
                       (Precision.BF16X6, "grouped plan in a CUDA graph"),
                       (Precision.FP16X3, "grouped plan in a CUDA graph")):
        tuned = None
        if prec != Precision.FP32:  # the grouped autotuner picks the tile configuration for this problem class
            tuned = ctx.autotune_grouped(prec, descs, reps=3)
        plan = ctx.grouped_plan(prec, descs)
        reset_c()
        ctx.grouped_run(plan)
        ctx.synchronize()
        err = errors()
        graph = None
        if prec != Precision.FP32:
            ctx.graph_begin()
            ctx.grouped_run(plan)
            graph = ctx.graph_end()

        def step():
            if graph is not None:
                ctx.graph_launch(graph)
            else:
                ctx.grouped_run(plan)
        for _ in range(args.warmup):
            step()
        ctx.synchronize()
        e0, e1 = ctx.event(), ctx.event()
        e0.record()
        for _ in range(args.steps):
            step()
        e1.record()
        ctx.synchronize()
        ms = e0.elapsed_ms(e1) / args.steps
        # one more eager run with per-kernel events: where the step's time goes
        ctx.profile_read()
        ctx.profile(True)
        ctx.grouped_run(plan)
        ctx.synchronize()
        ctx.profile(False)
        kern = {k: round(t / c, 4) for k, (c, t) in ctx.profile_read().items()}
        out[prec.name.lower()] = {"mode": mode, "ms_per_step": ms, "tflops": flops / (ms * 1e-3) / 1e12, **err,
                                  "launches_per_step": 2 if graph is not None else count,
                                  "kernel_ms_eager": kern if graph is not None else
                                  {"sgemm (all launches)": round(sum(kern.values()), 4)}}
        if tuned is not None:
            out[prec.name.lower()]["tile_config"] = ctx.grouped_config_of(plan)
            out[prec.name.lower()]["autotune_best_ms"] = tuned[1]
        if graph is not None:
            ctx.graph_destroy(graph)
        ctx.grouped_destroy(plan)
    out["speedup_bf16x3_vs_fp32"] = out["bf16x3"]["tflops"] / out["fp32"]["tflops"]

    # the members HBM bounds: K <= 128 (C read and written per call against 2 M N K
    # FLOPs), as a grouped plan of their own against their per-GEMM FP32 launches
    sub = [i for i, (M, N, K) in enumerate(shapes) if K <= 128]
    sub_bytes = float(sum(4 * (M * K + K * N + 2 * M * N) for M, N, K in (shapes[i] for i in sub)))
    peaks, _ = load_peaks()
    hbm = peaks.get("hbm_gbs")
    small = {"count": len(sub), "bytes_per_step": sub_bytes,
             "bytes": "sum of 4 (M K + K N + 2 M N): A, B read, C read and written"}
    sub_descs = ctx.descs([items[i] for i in sub])
    for prec in (Precision.FP32, Precision.BF16X3):
        if prec != Precision.FP32:
            ctx.autotune_grouped(prec, sub_descs, reps=3)
        plan = ctx.grouped_plan(prec, sub_descs)
        graph = None
        if prec != Precision.FP32:
            ctx.graph_begin()
            ctx.grouped_run(plan)
            graph = ctx.graph_end()

        def sub_step():
            if graph is not None:
                ctx.graph_launch(graph)
            else:
                ctx.grouped_run(plan)
        for _ in range(args.warmup):
            sub_step()
        ctx.synchronize()
        e0, e1 = ctx.event(), ctx.event()
        e0.record()
        for _ in range(args.steps):
            sub_step()
        e1.record()
        ctx.synchronize()
        ms = e0.elapsed_ms(e1) / args.steps
        gbs = sub_bytes / (ms * 1e-3) / 1e9
        small[prec.name.lower()] = {"ms_per_step": ms, "gbs": gbs, "frac_of_hbm": gbs / hbm if hbm else None}
        if prec != Precision.FP32:
            small[prec.name.lower()]["tile_config"] = ctx.grouped_config_of(plan)
        if graph is not None:
            ctx.graph_destroy(graph)
        ctx.grouped_destroy(plan)
    out["small_k_members"] = small
    for r in refs:
        ctx.free(r)
    for _, dA, dB, dC in mats:
        for b in (dA, dB, dC):
            ctx.free(b)
    return out


# ------------------------------------------------------------ CPU baseline
def cpu_gemm_sample(n: int, target_s: float) -> dict:
    """The reference kernel body (gemm.cpp:82-91) on the host cores through the
    oracle's port, on the first `rows` output rows, `rows` grown until one sample
    takes about `target_s` seconds."""
    sys.path.insert(0, str(ROOT / "oracle"))
    import oracle

    lib = oracle.fast_lib()
    A, B, C = polybench_gemm_init(n)
    rows = 1
    while True:
        t = time.perf_counter()
        lib.orc_gemm_body(A, B, C, n, 0, rows, ALPHA, BETA)
        dt = time.perf_counter() - t
        if dt >= target_s or rows >= n:
            break
        rows = min(n, max(rows * 2, int(rows * target_s / max(dt, 1e-3) * 0.9)))
    return {"rows": rows, "seconds": dt, "tflops": 2.0 * rows * n * n / dt / 1e12,
            "cores": lib.orc_num_threads()}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--size", type=int, default=8192)
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="target length of the CPU baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-grouped", action="store_true", help="skip the grouped 512-GEMM workload")
    ap.add_argument("--grouped-count", type=int, default=512)
    ap.add_argument("--no-family", action="store_true", help="skip the 2mm/3mm/syrk/syr2k section")
    ap.add_argument("--no-small-k", action="store_true", help="skip the small-K (HBM-bound) GEMM section")
    ap.add_argument("--no-neighbours", action="store_true",
                    help="skip covariance/correlation/matmulchain/matrix-vector section")
    ap.add_argument("--forms", default="fp32,bf16x3,tf32x3,bf16x6,fp16x3,tf32,fp8", help="forms to time (comma list)")
    ap.add_argument("--tile-config", type=int, default=None, help="force this tile configuration (no autotuning)")
    ap.add_argument("--family-size", type=int, default=4096)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    dist = Dist()
    n = args.size
    config = {"workload": f"polybench gemm C=alpha*A*B+beta*C, N={n} (NI=NJ=NK), alpha=32412, beta=2123, "
                          f"polybench init A=i*k/N B=(k*j+1)/N C=(i*j+2)/N",
              "size": n, "flops_per_step": 2 * n ** 3, "l2": "inputs larger than L2 (3 x N^2 x 4 B), no flush; C restored from its initial copy before "
                                "every step, outside the step's events",
              "parallelism": f"replicas x{dist.world}"}
    base = {"metric": "GEMM-family TFLOP/s (split-BF16 tcgen05 vs plain FP32 SIMT, matched FP64 error)",
            "unit": "TFLOP/s", "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "data": "synthetic (analytic polybench init)",
            "config": config}

    if args.impl == "reference":
        if dist.rank != 0:
            dist.close()
            return
        samples = []
        for s in range(args.warmup + args.steps):
            r = cpu_gemm_sample(n, min(args.cpu_seconds, 8.0))
            if s >= args.warmup:
                samples.append(r)
        best = max(samples, key=lambda r: r["tflops"])
        val = statistics.median(r["tflops"] for r in samples)
        line = dict(base, impl="reference", value=val, ms_per_step=statistics.median(
            r["seconds"] * 1e3 for r in samples), dtype="f32",
            cpu_baseline={"value": val, "unit": "TFLOP/s", "cores": best["cores"], "kind": "port",
                          "sample": f"first {best['rows']} of {n} output rows of the gemm.cpp:82-91 kernel body, "
                                    f"OpenMP over (row, 64-wide column block), -O3 -ffast-math"},
            e2e={"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0})
        print(json.dumps(line))
        dist.close()
        return

    res = run_gpu(args, dist)
    cpu = None
    if dist.rank == 0 and dist.world == 1 and not args.no_cpu_baseline:
        r = cpu_gemm_sample(n, args.cpu_seconds)
        cpu = {"value": r["tflops"], "unit": "TFLOP/s", "cores": r["cores"], "kind": "port",
               "sample": f"first {r['rows']} of {n} output rows of the gemm.cpp:82-91 kernel body on the host "
                         f"cores ({r['seconds']:.1f} s), oracle port built -O3 -ffast-math"}
    if dist.rank == 0:
        line = dict(base, value=res["value"], ms_per_step=res["ms_per_step"],
                    dtype=DTYPE_OF_FORM[res["headline"]],
                    e2e=res["e2e"], roofline=res["roofline"], cpu_baseline=cpu, clocks=res["clocks"],
                    err_vs_fp64=res["err_vs_fp64"], matched_error=res["matched_error"],
                    gpu_launches=res["gpu_launches"], tiers=res["tiers"], headline_form=res["headline"],
                    device={"sm_count": res["device"]["sm_count"], "cc": list(res["device"]["cc"])},
                    peaks=res["peak_kind"], grouped=res["grouped"], family=res["family"],
                    neighbours=res["neighbours"], small_k=res["small_k"])
        print(json.dumps(line))
    dist.close()


if __name__ == "__main__":
    main()

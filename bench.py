"""Benchmark of the GB300 GGKS bucket multiselect.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ggks|reference]

Workload (one "step"): one exact multiselect of a resident 2^28-element float32
vector drawn from normal(0,1) (seed 1) with 1001 distinct k's drawn uniformly
from [1, n] -- the large single-multiselect configuration.  The other inputs of
that configuration (Cauchy, half-normal, uint32, float64) and the top-k
configuration (2^26 float32 uniform, uint32 over 2^16 values and an ascending
float32 copy; K = 32, 1024, 65536) are timed after the headline and reported
under "variants".

Metric: input GB/s per multiselect = n * sizeof(T) / time of one wrapper call
(k upload, all passes, result download, synchronisation).  "e2e" is the same
metric through the host-vector entry point with the 1 GiB vector in pinned host
memory, so the host-to-device copy is inside every step.

"variants.reference_gpu": the reference's own kernels (built for sm_103a from
its sources, oracle/ref_gpu.py) under a restatement of its host code, timed on
this GPU as its timing adapter times them, on the headline input, the plain
configuration and the float32 top-k input, beside this path's calls; their
answers are compared with this path's.

"batched": the batched workload -- 4096 resident float32 vectors of log-uniform
lengths in [2^10, 2^22] with 1-64 k's each -- selected by one batched call (one
persistent launch), against 4096 sequential ggks_multiselect_f32 calls on the
same vectors (requests/s, bit-exact comparison).

"served": Poisson request streams at 1k-50k requests/s (and 100k, above that
range, for the server's capacity) through a ggks_server against sequential
plain calls (requests/s, p50/p99 latency, bit-exact comparison).

Under torchrun (N > 1) every rank runs an independent replica on its own GPU
(the path does not shard: replicas only); value = all ranks' bytes / max time.

--impl reference times the reference's sort-and-choose path (its own oracle,
multiselectTimingFunctions.cu:51-95) restated on the CPU (oracle/), with all
host threads, on the same workload; rank 0 only.
"""
import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "ggks-multiselect_gb300"))

N_LOG2 = 28
NUM_K = 1001
METRIC = "input GB/s per multiselect (2^28 f32 normal, 1001 k's)"
PEAK_FALLBACK_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ggks", choices=["ggks", "reference"])
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batched", action="store_true")
    ap.add_argument("--no-served", action="store_true")
    ap.add_argument("--only", choices=["batched", "served"], default=None,
                    help="run one section alone and print it as its own JSON line (profiling)")
    ap.add_argument("--batch-problems", type=int, default=4096)
    ap.add_argument("--log2n", type=int, default=N_LOG2)
    return ap.parse_args()


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return PEAK_FALLBACK_GBS, "fallback"


def workload(log2n):
    """The headline input: the large configuration's float32 normal vector
    (seed 1) with its 1001 distinct k's (seed 101)."""
    import ggks_problems as gp
    return gp.config_l("f32_normal", log2n)


def bench_config(log2n, ws):
    """The workload's description, printed identically by both arms."""
    n = 1 << log2n
    return {"workload": f"multiselect n=2^{log2n} f32 normal(0,1) seed 1, "
                        f"{NUM_K} distinct k's uniform in [1,n] (seed 101)",
            "n": n, "num_k": NUM_K, "elem": "float32 (ordered as u32 keys)",
            "parallelism": "replicas" if ws > 1 else "single GPU",
            "l2": (f"input ({n * 4 >> 20} MiB) larger than L2 (129 MB); no flush needed"
                   if n * 4 > 129 * 10**6 else
                   f"input ({n * 4 >> 20} MiB) smaller than L2 (129 MB): not flushed")}


def same_bits(a, b):
    a, b = np.ascontiguousarray(a), np.ascontiguousarray(b)
    return a.dtype == b.dtype and a.shape == b.shape and bool(
        np.array_equal(a.view(np.uint8), b.view(np.uint8)))


# ---------------------------------------------------------------------------
# clocks: NVML through ctypes (reading only), nvidia-smi as a fallback
# ---------------------------------------------------------------------------
REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
           0x40: "hw_thermal_slowdown", 0x80: "hw_power_brake_slowdown"}


class ClockSampler:
    def __init__(self, index, period=0.01):
        self.samples = []  # (t, sm_mhz, reasons_mask)
        self.period = period
        self.max_mhz = None
        self._stop = threading.Event()
        self._nvml = None
        self._h = None
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() == 0:
                h = ctypes.c_void_p()
                if nv.nvmlDeviceGetHandleByIndex_v2(int(index), ctypes.byref(h)) == 0:
                    self._nvml, self._h = nv, h
                    m = ctypes.c_uint()
                    if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(m)) == 0:
                        self.max_mhz = m.value
        except OSError:
            pass
        self._thr = threading.Thread(target=self._run, daemon=True)

    def _one(self):
        nv, h = self._nvml, self._h
        c = ctypes.c_uint()
        r = ctypes.c_ulonglong()
        if nv.nvmlDeviceGetClockInfo(h, 1, ctypes.byref(c)) != 0:
            return None
        fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            nv.nvmlDeviceGetCurrentClocksThrottleReasons
        if fn(h, ctypes.byref(r)) != 0:
            r.value = 0
        return c.value, r.value

    def _run(self):
        while not self._stop.is_set():
            if self._nvml is not None:
                s = self._one()
                if s:
                    self.samples.append((time.perf_counter(), s[0], s[1]))
            time.sleep(self.period)

    def start(self):
        if self._nvml is not None:
            self._thr.start()
        return self

    def stop(self):
        self._stop.set()
        if self._thr.is_alive():
            self._thr.join()

    def summary(self, t0, t1):
        inside = [s for s in self.samples if t0 <= s[0] <= t1]
        src = "nvml"
        if not inside:
            # region shorter than the sampling period: nearest samples
            inside = sorted(self.samples, key=lambda s: min(abs(s[0] - t0), abs(s[0] - t1)))[:3]
            src = "nvml (nearest samples; timed region shorter than the sampling period)"
        if not inside:
            return self._smi_fallback()
        mask = 0
        for s in inside:
            mask |= s[2]
        return {"sm_mhz": statistics.median(s[1] for s in inside), "sm_max_mhz": self.max_mhz,
                "reasons": [v for b, v in REASONS.items() if mask & b], "samples": len(inside),
                "source": src}

    def _smi_fallback(self):
        try:
            out = subprocess.run(["nvidia-smi", "--query-gpu=clocks.sm,clocks.max.sm",
                                  "--format=csv,noheader,nounits"], capture_output=True,
                                 text=True, timeout=20).stdout.strip().splitlines()[0]
            sm, mx = [float(v) for v in out.split(",")]
            return {"sm_mhz": sm, "sm_max_mhz": mx, "reasons": [], "samples": 1,
                    "source": "nvidia-smi after the run"}
        except Exception:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0,
                    "source": "unavailable"}


# ---------------------------------------------------------------------------
# reference arm: the CPU sort-and-choose path, all host threads, rank 0 only
# ---------------------------------------------------------------------------
def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    x, k = workload(args.log2n)
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        oracle.multiselect(x, k, threads=threads)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        oracle.multiselect(x, k, threads=threads)
        times.append(time.perf_counter() - t0)
    t = sum(times) / len(times)
    gbs = x.nbytes / t / 1e9
    line = {
        "impl": "reference", "metric": METRIC, "value": round(gbs, 4), "unit": "GB/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(t * 1e3, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "u32", "data": "synthetic",
        "config": bench_config(args.log2n, ws),
        "cpu_baseline": {"value": round(gbs, 4), "unit": "GB/s", "cores": threads, "kind": "port",
                         "sample": f"full workload per step: sort-and-choose of all {x.size} "
                                   f"elements, {threads} threads (parallel LSD radix sort of keys)"},
        "e2e": {"value": round(gbs, 4), "unit": "GB/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# our arm
# ---------------------------------------------------------------------------
def cpu_baseline(x, k):
    """Single-threaded sort-and-choose with std::sort (the reference's own
    oracle, multiselectTimingFunctions.cu:51-95, on the host) on a bounded
    sample of the workload: the first 2^26 elements with the k list clipped to
    that length."""
    orc = oracle_mod()
    m = 1 << 26
    xs = x[:m]
    ks = np.clip(k, 1, m).astype(np.uint32)
    t0 = time.perf_counter()
    orc.multiselect_stdsort(xs, ks)
    dt = time.perf_counter() - t0
    return {"value": round(xs.nbytes / dt / 1e9, 4), "unit": "GB/s", "cores": 1, "kind": "port",
            "sample": f"first 2^26 of the 2^28 elements (256 MiB), {ks.size} k's clipped to "
                      f"[1, 2^26]: one single-threaded std::sort of the keys, then index "
                      f"({dt:.2f} s)"}


def timed_steps(fn, steps, warmup, stream, torch, after_warmup=None):
    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    if after_warmup:
        after_warmup()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        ev0.record(stream)
        t0 = time.perf_counter()
        for _ in range(steps):
            fn()
        ev1.record(stream)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    return ev0.elapsed_time(ev1) / steps, t0, t1


def run_ggks(args):
    import torch
    import torch.distributed as dist

    import ggks
    import ggks_problems as gp

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    x, k = workload(args.log2n)
    n = x.size
    d_x = torch.from_numpy(x).to(dev)
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    ctx = ggks.Context(local)
    out = np.empty(k.size, dtype=np.float32)

    def step():
        ggks.multiselect_ptr(d_x.data_ptr(), n, np.float32, k, ctx=ctx, stream=sptr, out=out)

    sampler = ClockSampler(local).start()
    if ws > 1:
        dist.barrier()
    torch.cuda.synchronize()
    # every pass's device time first: steps with CUDA events around every pass
    # (they also pick the dominant streaming pass, the roofline's kernel),
    # for at least half a second, so that the SM clock has settled at its
    # steady value before the timed steps (a cold GPU starts ~4 % lower)
    ctx.set_profiling(True)
    ctx.reset_stats()
    t_pre = time.perf_counter()
    done = 0
    while done < 3 or time.perf_counter() - t_pre < 0.5:
        step()
        done += 1
    torch.cuda.synchronize()
    st_all = ctx.stats()
    pass_ms = {p: st_all["pass_ms"][p] / max(1, st_all["pass_launches"][p]) for p in ggks.PASS_NAMES}
    dom = max(("hist", "compact"), key=lambda p: pass_ms[p])
    # a vector small enough for the one-launch path has a single kernel
    # (k_small), timed as the sample pass
    small_path = st_all["small_calls"] > 0 and pass_ms[dom] == 0.0
    if small_path:
        dom = "sample"
    # inside the timed region CUDA events bracket the dominant pass only (an
    # event between two kernels gives up their overlapped launch); launch
    # counts cover the timed steps only
    ctx.set_profiling(True, passes=(dom,))
    ms, t0, t1 = timed_steps(step, args.steps, args.warmup, stream, torch,
                             after_warmup=ctx.reset_stats)
    st = ctx.stats()
    ctx.set_profiling(False)
    timed_out = out.copy()  # the last timed call's answers, checked below
    gpu_launches = int(st["launches"])
    stream_ms = {dom: st["pass_ms"][dom] / max(1, st["pass_launches"][dom])}
    clocks = sampler.summary(t0, t1)
    tmax = torch.tensor([ms], dtype=torch.float64, device=dev)
    if ws > 1:
        dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
        dist.barrier()
    ms_max = float(tmax.item())
    value = ws * n * 4 / (ms_max * 1e-3) / 1e9

    peak, peak_kind = measured_peak()
    achieved = n * 4 / (stream_ms[dom] * 1e-3) / 1e9
    traffic = read_traffic("small" if small_path else dom)
    roofline = {"bound": "hbm", "kernel": "k_small" if small_path else f"k_{dom}",
                "achieved": round(achieved, 1),
                "peak": peak, "unit": "GB/s", "frac": round(achieved / peak, 4),
                "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind ==
                "measured" else "fallback 6.8 TB/s",
                "traffic": traffic,
                "algorithmic_bytes_per_launch": n * 4,
                "whole_call_frac": round(value / ws / peak, 4)}

    # e2e: host vector (pinned) -> device copy inside every step
    h_pin = torch.empty(n, dtype=torch.float32, pin_memory=True)
    h_pin.numpy()[:] = x
    hx = h_pin.numpy()

    def e2e_step():
        ggks.multiselect_host(hx, k, ctx=ctx, stream=sptr, out=out)

    e2e_steps = max(3, min(args.steps, 20))
    e2e_ms, _, _ = timed_steps(e2e_step, e2e_steps, 2, stream, torch)
    etmax = torch.tensor([e2e_ms], dtype=torch.float64, device=dev)
    if ws > 1:
        dist.all_reduce(etmax, op=dist.ReduceOp.MAX)
    e2e_val = ws * n * 4 / (float(etmax.item()) * 1e-3) / 1e9
    sampler.stop()
    # the timed calls' answers against sort-and-choose (outside every timed
    # region): the headline on every rank, the rest on rank 0 below
    want = oracle_mod().multiselect(x, k, threads=os.cpu_count() or 1)
    parity = {"headline": same_bits(timed_out, want), "headline_e2e": same_bits(out, want)}

    variants = {}
    if not args.no_variants and rank == 0:
        variants = run_variants(torch, ggks, gp, ctx, stream, sptr, dev, args.log2n, parity)
        variants["reference_gpu"] = run_reference_gpu(torch, ggks, gp, dev, x, k, ms_max,
                                                      parity)
    batched = served = None
    if not args.no_batched and rank == 0:
        batched = run_batched(torch, ggks, gp, dev, sptr)
    if not args.no_served and rank == 0:
        served = run_served(torch, ggks, gp, dev, sptr)

    if rank == 0:
        line = {
            "metric": METRIC.replace("2^28", f"2^{args.log2n}"), "value": round(value, 2),
            "unit": "GB/s", "n_gpus": ws,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max, 4),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (numpy PCG64)",
            "config": bench_config(args.log2n, ws),
            "elements_per_s": round(ws * n / (ms_max * 1e-3), 1),
            "roofline": roofline,
            "pass_ms": {p: round(v, 4) for p, v in pass_ms.items()},
            "survivors_per_call": int(st["survivors"] // max(1, st["calls"])),
            "recursions_per_call": round(st["recursions"] / max(1, st["calls"]), 3),
            "e2e": {"value": round(e2e_val, 2), "unit": "GB/s",
                    "h2d_bytes_per_step": n * 4 + k.size * 4, "d2h_bytes_per_step": k.size * 4,
                    "entry": "ggks_multiselect_host_f32 (pinned host vector)"},
            "gpu_launches": gpu_launches,
            "clocks": clocks,
            "parity": all(parity.values()),
            "parity_checked": {kk: bool(v) for kk, v in parity.items()},
        }
        if variants:
            line["variants"] = variants
        if batched:
            line["batched"] = batched
        if served:
            line["served"] = served
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(x, k)
        print(json.dumps(line), flush=True)
    ctx.close()
    if ws > 1:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def oracle_mod():
    """The CPU checker (sort-and-choose), used outside every timed region."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    return oracle


def timed_calls_flushed(fn, steps, warmup, stream, torch, dev):
    """Per-call device time of a synchronous call on a small input: before
    each call a 256 MiB write evicts the input from L2 (129 MB); CUDA events
    bracket only the call.  Returns the mean ms per call."""
    flush = torch.empty(64 << 20, dtype=torch.float32, device=dev)
    for _ in range(warmup):
        fn()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
          for _ in range(steps)]
    with torch.cuda.stream(stream):
        for e0, e1 in ev:
            flush.zero_()
            e0.record(stream)
            fn()
            e1.record(stream)
    torch.cuda.synchronize()
    return sum(e0.elapsed_time(e1) for e0, e1 in ev) / steps


def run_variants(torch, ggks, gp, ctx, stream, sptr, dev, log2n, parity):
    """The other inputs of the large configuration, the top-k configuration
    and the plain configuration, timed the same way; each timed call's answers
    are checked against sort-and-choose outside the timed regions."""
    orc = oracle_mod()
    thr = os.cpu_count() or 1
    res = {}
    for name, dt, dist_name, lg, seed in gp.L_INPUTS[1:]:
        lg = lg - (N_LOG2 - log2n)
        x, k = gp.config_l(name, lg)
        n = x.size
        carrier = x.view(np.int32) if dt == "u32" else x
        d = torch.from_numpy(carrier).to(dev)
        out = np.empty(k.size, dtype=x.dtype)

        def step():
            ggks.multiselect_ptr(d.data_ptr(), n, x.dtype, k, ctx=ctx, stream=sptr, out=out)

        ms, _, _ = timed_steps(step, 10, 3, stream, torch)
        parity[name] = same_bits(out, orc.multiselect(x, k, threads=thr))
        res[name] = {"n": n, "ms": round(ms, 4), "GB/s": round(x.nbytes / (ms * 1e-3) / 1e9, 1)}
        del d
    # top-k configuration: K in {32, 1024, 65536} on 2^26 float32 uniform,
    # uint32 uniform over [0, 2^16) and the ascending float32 copy (ms per call)
    n = 1 << gp.T_LOG2N
    grid = {}
    detail = None
    for name in gp.T_INPUTS:
        x = gp.config_t(name)
        carrier = x.view(np.int32) if x.dtype == np.uint32 else x
        d = torch.from_numpy(carrier).to(dev)
        want = orc.topk(x, max(gp.T_KS), threads=thr)
        row = {}
        for K in gp.T_KS:
            o = np.empty(K, dtype=x.dtype)

            def tkk():
                ggks.topk_ptr(d.data_ptr(), n, x.dtype, K, ctx=ctx, stream=sptr, out=o)

            ms, _, _ = timed_steps(tkk, 10, 3, stream, torch)
            parity[f"topk_{name}_K{K}"] = same_bits(o, want[:K])
            row[str(K)] = round(ms, 4)
        grid[name] = row
        if name == "f32_uniform":
            # per-pass device times of the K = 65536 call (events around every pass)
            ctx.set_profiling(True)
            ctx.reset_stats()
            o = np.empty(65536, dtype=x.dtype)
            for _ in range(5):
                ggks.topk_ptr(d.data_ptr(), n, x.dtype, 65536, ctx=ctx, stream=sptr, out=o)
            torch.cuda.synchronize()
            st = ctx.stats()
            ctx.set_profiling(False)
            detail = {"n": n, "ms": row["65536"],
                      "GB/s": round(x.nbytes / (row["65536"] * 1e-3) / 1e9, 1),
                      "pass_ms": {p: round(st["pass_ms"][p] / max(1, st["pass_launches"][p]), 4)
                                  for p in ggks.PASS_NAMES},
                      "recursions": st["recursions"], "survivors": st["survivors"] // 5}
        del d
    res["topk_f32_2^26_K65536"] = detail
    res["topk_grid_2^26_ms"] = grid
    # plain configuration: 2^20 float32 uniform (seed 0), 101 k's on the p grid;
    # the 4 MiB input fits L2, so L2 is flushed before every timed call
    x, k = gp.config_p()
    d = torch.from_numpy(x).to(dev)
    out = np.empty(k.size, dtype=x.dtype)

    def pstep():
        ggks.multiselect_ptr(d.data_ptr(), x.size, x.dtype, k, ctx=ctx, stream=sptr, out=out)

    ms = timed_calls_flushed(pstep, 50, 5, stream, torch, dev)
    parity["plain_P"] = same_bits(out, orc.multiselect(x, k, threads=thr))
    res["plain_P_2^20_101k"] = {"n": x.size, "num_k": int(k.size), "us": round(ms * 1e3, 2),
                                "GB/s": round(x.nbytes / (ms * 1e-3) / 1e9, 1),
                                "l2": "flushed before every call (256 MiB write, not timed)"}
    del d
    return res


def run_reference_gpu(torch, ggks, gp, dev, x, k, ours_ms, parity):
    """The reference's own bucket multiselect on this GPU: its kernels
    (bucketMultiselect.cu, compiled for sm_103a from its sources) under a
    restatement of its host code (oracle/ref_gpu.py), on the headline input,
    the plain configuration and the top-k configuration's float32 input.
    Each call is timed as timeBucketMultiselect times it
    (multiselectTimingFunctions.cu:100-122: CUDA events on the legacy stream
    around the wrapper, its allocations and copies included), on a resident
    vector; ``ours`` is this path's call on the same input.  The answers are
    compared with this path's, outside the timed calls."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import ref_gpu
    why = ref_gpu.unavailable()
    if why:
        return {"unavailable": why}
    ref_gpu.lib()
    sms, mt = ref_gpu.device_shape()

    def ref_calls(xv, kv, reps):
        p = ref_gpu.padded_device_copy(xv)
        ref_gpu.bucket_multiselect_device(p.data_ptr(), xv.size, kv, xv.dtype)  # warm-up
        times, outs = [], None
        for _ in range(reps):
            outs, ms = ref_gpu.bucket_multiselect_device(p.data_ptr(), xv.size, kv, xv.dtype)
            times.append(ms)
        del p
        torch.cuda.empty_cache()
        return outs, statistics.median(times)

    def ours_call(xv, kv, topk=None, reps=10):
        carrier = xv.view(np.int32) if xv.dtype == np.uint32 else xv
        d = torch.from_numpy(carrier).to(dev)
        ctx = ggks.Context(dev.index or 0)

        def f():
            if topk:
                return ggks.topk_ptr(d.data_ptr(), xv.size, xv.dtype, topk, ctx=ctx)
            return ggks.multiselect_ptr(d.data_ptr(), xv.size, xv.dtype, kv, ctx=ctx)

        for _ in range(3):
            f()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        times = []
        for _ in range(reps):
            e0.record()
            o = f()
            e1.record()
            e1.synchronize()
            times.append(e0.elapsed_time(e1))
        ctx.close()
        del d
        return o, statistics.median(times)

    res = {"kernels": "the reference's own (bucketMultiselect.cu:129-325) built for sm_103a",
           "host": "phaseOne / generatePivots / bucketMultiselectWrapper restated "
                   "(bucketMultiselect.cu:414-871), same launches, copies and allocations",
           "launch_shape": {"blocks": sms, "threads": mt},
           "timing": "CUDA events around one wrapper call on a resident vector (median); "
                     "ours: the same around one synchronous call of this path"}
    out, ms = ref_calls(x, k, 5)
    ours, _ = ours_call(x, k, reps=3)
    parity["reference_gpu_headline"] = same_bits(out, ours)
    res["headline"] = {"n": x.size, "num_k": int(k.size), "ms": round(ms, 3),
                       "GB/s": round(x.nbytes / (ms * 1e-3) / 1e9, 1), "ours_ms": round(ours_ms, 4),
                       "speedup": round(ms / ours_ms, 1)}
    xp, kp = gp.config_p()
    out, ms = ref_calls(xp, kp, 20)
    ours, oms = ours_call(xp, kp, reps=20)
    parity["reference_gpu_plain_P"] = same_bits(out, ours)
    res["plain_P_2^20_101k"] = {"ms": round(ms, 3), "ours_ms": round(oms, 4),
                                "speedup": round(ms / oms, 1)}
    xt = gp.config_t("f32_uniform")
    topk = {}
    for K in gp.T_KS:
        out, ms = ref_calls(xt, np.arange(1, K + 1, dtype=np.uint32), 5)
        ours, oms = ours_call(xt, None, topk=K)
        parity[f"reference_gpu_topk_K{K}"] = same_bits(out, ours)
        topk[str(K)] = {"ms": round(ms, 3), "ours_ms": round(oms, 4),
                        "speedup": round(ms / oms, 1)}
    res["topk_f32_uniform_2^26"] = topk
    return res


def run_batched(torch, ggks, gp, dev, sptr, count=4096):
    """The batched workload: `count` float32 vectors with log-uniform lengths
    in [2^10, 2^22], four distributions, 1-64 k's each (seed 1), resident on
    the device.  One batched call (one persistent launch) against `count`
    sequential ggks_multiselect_f32 calls on the same vectors; outputs are
    compared bit for bit."""
    probs = gp.batch_problems(count, seed=1)
    vecs = gp.batch_vectors_device(probs, seed=1, device=dev)
    torch.cuda.synchronize()
    ptrs = [v.data_ptr() for v in vecs]
    ns = [v.numel() for v in vecs]
    ks = [np.ascontiguousarray(p["k"], dtype=np.uint32) for p in probs]
    total = int(sum(ns))
    reqs = int(sum(k.size for k in ks))
    ctx = ggks.Context(dev.index or 0)
    b = ggks.PreparedBatch(ptrs, ns, np.float32, ks, ctx=ctx, stream=sptr, autotune=True)
    t0 = time.perf_counter()
    b()  # first call of this batch shape: the autotuner times every candidate
    tune_s = time.perf_counter() - t0
    batch_out = b().copy()
    ctx.reset_stats()
    wall = []
    for _ in range(7):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        b()
        wall.append(time.perf_counter() - t0)
    st = ctx.stats()
    calls = max(1, st["batch_calls"])
    phase_ms = {k: round(v / calls, 4) for k, v in st["batch_phase_ms"].items()}
    t_batch = statistics.median(wall)

    # sequential plain calls on the same resident vectors
    L = ggks.lib()
    f = L.ggks_multiselect_f32
    o = ggks._opts(ctx, sptr)
    outs = [np.empty(k.size, dtype=np.float32) for k in ks]
    args_list = [(ctypes.c_void_p(p), int(n), k.ctypes.data, k.size, out.ctypes.data)
                 for p, n, k, out in zip(ptrs, ns, ks, outs)]
    for a in args_list[:32]:
        f(*a, ctypes.byref(o))
    torch.cuda.synchronize()
    seq = []
    for _ in range(2):
        t0 = time.perf_counter()
        for a in args_list:
            st_ = f(*a, ctypes.byref(o))
            if st_ != 0:
                raise RuntimeError(f"plain call failed: {st_}")
        seq.append(time.perf_counter() - t0)
    t_seq = min(seq)
    exact = all(np.array_equal(a.view(np.uint32), c.view(np.uint32))
                for a, c in zip(b.split(batch_out), outs))
    tune = ggks.batch_last_tuning(ctx)
    ctx.close()
    del vecs
    torch.cuda.empty_cache()
    return {
        "workload": f"{count} float32 vectors, lengths log-uniform in [2^10, 2^22] (seed 1), "
                    "distributions uniform[0,1) / normal(0,1) / Cauchy / integer-valued "
                    "[0,256), 1-64 k's each uniform in [1, len]; resident in HBM",
        "problems": count, "elements": total, "outputs": reqs,
        "req_per_s": round(count / t_batch, 1), "ms_per_batch": round(t_batch * 1e3, 3),
        "GB/s": round(total * 4 / t_batch / 1e9, 1),
        "kernel_ms": round(sum(phase_ms.values()), 3), "phase_ms": phase_ms,
        "launches_per_batch": round(st["launches"] / calls, 2), "ctas": st["batch_grid"],
        "survivors_per_batch": int(st["survivors"] // calls),
        "recursions_per_batch": round(st["recursions"] / calls, 2),
        "tuning": {"div": tune[0], "tile": tune[1], "autotune_s": round(tune_s, 3)},
        "sequential_plain": {"ms": round(t_seq * 1e3, 2), "req_per_s": round(count / t_seq, 1),
                             "entry": "ggks_multiselect_f32, one call per vector"},
        "speedup_req_per_s": round(t_seq / t_batch, 2),
        "bit_exact_vs_plain": bool(exact),
        "timing": "host wall clock per call (synchronous C-ABI call: planning, upload, launch, "
                  "results); median of 7",
    }


# 1k-50k requests/s is the serving configuration's range.  At 50k the trace
# itself caps the served rate near 48k, so the ratio there is bounded by 50k over
# the sequential rate; 100k, above the range, shows the server's capacity.
SERVE_RATES = (1000, 5000, 20000, 50000, 100000)
# requests per rate: 4000, and 12000 at the capacity point above the
# configuration's range (with 4000, about 13 batches, one batch boundary
# moved the measured capacity by up to 15 % between runs)
SERVE_REQUESTS = {100000: 12000}


def run_served(torch, ggks, gp, dev, sptr, per_rate=4000):
    """The served workload: Poisson arrivals at each rate of SERVE_RATES over
    a resident pool of mixed vectors (float32 : uint32 : float64 = 6 : 3 : 1,
    lengths log-uniform in [2^12, 2^26]); 70% multiselects with 8-1024 k's,
    30% top-k with K in [16, 4096]; HBM admission cap 64 GB.  The served arm
    submits every request at its arrival time to a ggks_server (continuous
    batching); the sequential arm runs plain calls in arrival order, each
    starting at its arrival time or when the previous one returns.  Latency =
    completion - scheduled arrival."""
    DT = {"f32": np.float32, "u32": np.uint32, "f64": np.float64}
    pool = gp.serving_pool({"f32": 48, "u32": 24, "f64": 8}, seed=7, device=dev)
    torch.cuda.synchronize()
    sizes = {dt: [v.numel() for v in vs] for dt, vs in pool.items()}
    ptrs = {dt: [v.data_ptr() for v in vs] for dt, vs in pool.items()}
    L = ggks.lib()
    ctx = ggks.Context(dev.index or 0)
    o = ggks._opts(ctx, sptr)
    fms = {dt: getattr(L, "ggks_multiselect_" + dt) for dt in DT}
    ftk = {dt: getattr(L, "ggks_topk_" + dt) for dt in DT}

    def pct(a, q):
        return round(float(np.percentile(np.asarray(a) * 1e3, q)), 3)

    out = {"workload": "Poisson arrivals; requests 70% multiselect (8-1024 k's) / 30% top-k "
                       "(K in [16,4096]); float32:uint32:float64 = 6:3:1 over a resident pool "
                       "of 80 vectors, lengths log-uniform in [2^12, 2^26], mixed distributions; "
                       "HBM admission cap 64 GB",
           "requests_per_rate": {str(r): SERVE_REQUESTS.get(r, per_rate) for r in SERVE_RATES},
           "rates": {}}
    all_exact = True
    for rate in SERVE_RATES:
        trace = gp.serving_trace(sizes, rate, SERVE_REQUESTS.get(rate, per_rate), seed=rate)
        bufs = []
        for q in trace:
            num = q["K"] if q["k"] is None else q["k"].size
            bufs.append((np.empty(num, dtype=DT[q["dtype"]]), np.empty(num, dtype=DT[q["dtype"]])))
        in_bytes = sum(sizes[q["dtype"]][q["vec"]] * np.dtype(DT[q["dtype"]]).itemsize for q in trace)

        # ---- sequential plain calls
        seq_lat = []
        t0 = time.perf_counter() + 0.01
        for q, (so, _) in zip(trace, bufs):
            ta = t0 + q["t"]
            while time.perf_counter() < ta:
                pass
            dt = q["dtype"]
            p, n = ptrs[dt][q["vec"]], sizes[dt][q["vec"]]
            if q["k"] is None:
                st = ftk[dt](ctypes.c_void_p(p), n, q["K"], so.ctypes.data, ctypes.byref(o))
            else:
                st = fms[dt](ctypes.c_void_p(p), n, q["k"].ctypes.data, q["k"].size,
                             so.ctypes.data, ctypes.byref(o))
            if st != 0:
                raise RuntimeError(f"plain call failed: {st}")
            seq_lat.append(time.perf_counter() - ta)
        seq_span = (t0 + trace[-1]["t"] + seq_lat[-1]) - t0

        # ---- served: submit at arrival times, wait in order.  Every request
        # (its ggks_request, k list and output buffer) is built before the
        # clock starts, so the submitter only waits for each arrival time and
        # makes the C call: the offered rate is the trace's, not the rate at
        # which Python can build requests.
        srv = ggks.Server(dev.index or 0, hbm_cap_bytes=64 << 30)
        tickets = [None] * len(trace)
        sub_t = [0.0] * len(trace)
        sub_at = [0.0] * len(trace)
        prepared = []
        for i, q in enumerate(trace):
            dt = q["dtype"]
            karr = None if q["k"] is None else np.ascontiguousarray(q["k"], dtype=np.uint32)
            req = ggks.Request(ggks.DTYPE_CODES[np.dtype(DT[dt])],
                               ggks.REQ_TOPK if karr is None else 0,
                               ctypes.c_void_p(ptrs[dt][q["vec"]]), sizes[dt][q["vec"]],
                               karr.ctypes.data if karr is not None else None,
                               q["K"] if karr is None else karr.size, 0)
            prepared.append((req, karr, ctypes.c_void_p(bufs[i][1].ctypes.data),
                             ctypes.c_uint64()))
        fsub = L.ggks_server_submit

        def submitter():
            for i, q in enumerate(trace):
                ta = t1 + q["t"]
                while time.perf_counter() < ta:
                    pass
                req, _, optr, tk = prepared[i]
                now = time.perf_counter()
                sub_t[i] = now - ta
                sub_at[i] = now
                if fsub(srv.handle, ctypes.byref(req), optr, ctypes.byref(tk)) != 0:
                    raise RuntimeError("server submit failed")
                tickets[i] = tk.value

        t1 = time.perf_counter() + 0.01
        th = threading.Thread(target=submitter)
        th.start()
        srv_lat = [0.0] * len(trace)
        for i in range(len(trace)):
            while tickets[i] is None:
                time.sleep(50e-6)
            _, lat_ms = srv.wait(tickets[i])
            srv_lat[i] = sub_t[i] + lat_ms * 1e-3
        th.join()
        sst = srv.stats()
        srv.close()
        srv_span = max(q["t"] + lat for q, lat in zip(trace, srv_lat))
        sub_span = sub_at[-1] - sub_at[0]
        exact = all(np.array_equal(a.view(np.uint8), b.view(np.uint8)) for a, b in bufs)
        all_exact &= exact
        out["rates"][str(rate)] = {
            "offered_req_per_s": rate,
            "served": {"req_per_s": round(len(trace) / srv_span, 1),
                       "submitted_req_per_s": round((len(trace) - 1) / max(sub_span, 1e-9), 1),
                       "p50_ms": pct(srv_lat, 50), "p99_ms": pct(srv_lat, 99),
                       "GB/s": round(in_bytes / srv_span / 1e9, 1),
                       "batches": sst["batches"], "launches": sst["launches"],
                       "concurrent_launches": sst["concurrent_launches"],
                       "hbm_waits": sst["hbm_waits"], "single_calls": sst["single_calls"],
                       "recursions": sst["recursions"],
                       "batch_phase_ms": {p: round(v, 2) for p, v in sst["batch_phase_ms"].items()},
                       "kernel_ms": round(sst["kernel_ms"], 2),
                       "lane_group_ms": round(sst["group_ms"], 2),
                       "device_busy_ms": round(sst["device_busy_ms"], 2),
                       "device_span_ms": round(sst["device_span_ms"], 2),
                       "mean_batch": round(sst["batched_requests"] / max(1, sst["batches"]), 2)},
            "sequential_plain": {"req_per_s": round(len(trace) / seq_span, 1),
                                 "p50_ms": pct(seq_lat, 50), "p99_ms": pct(seq_lat, 99)},
            "req_per_s_ratio": round(seq_span / srv_span, 2),
            "bit_exact_vs_plain": bool(exact),
        }
    out["bit_exact_vs_plain"] = bool(all_exact)
    ctx.close()
    del pool
    torch.cuda.empty_cache()
    return out


def read_traffic(kernel):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/), scaled to the full workload there; None if absent."""
    p = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        for line in open(p):
            parts = line.split()
            if len(parts) >= 2 and parts[0] == f"k_{kernel}":
                return int(float(parts[1]))
    except OSError:
        pass
    return None


def run_section(args):
    """One section alone (for profiling): its object as one JSON line."""
    import torch

    import ggks
    import ggks_problems as gp
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    if args.only == "batched":
        res = run_batched(torch, ggks, gp, dev, stream.cuda_stream, count=args.batch_problems)
    else:
        res = run_served(torch, ggks, gp, dev, stream.cuda_stream)
    print(json.dumps({"section": args.only, args.only: res}), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        return run_section(args)
    return run_ggks(args)


if __name__ == "__main__":
    sys.exit(main())

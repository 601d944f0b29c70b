"""Benchmark: batched c32 DFT throughput on GB300 against the measured HBM roofline.

Workload (the mixed-radix / prime parity set): complex c32 DFT, forward, at
N in {1000, 1536, 2187, 30720, 127, 8191} with batch = 256 MiB / (8 N) signals each (33554, 21845, 15343,
1092, 264208, 4096).  One step = one forward pass over all six batches (1.5 GiB in, 1.5 GiB out); every
input is larger than L2, so no flush is needed between steps.  Inputs are seeded i.i.d. N(0,1) times a
seeded amplitude (synthetic; the reference publishes no dataset for this path).

value   = algorithmic bytes (16 N per signal: read N c32 + write N c32) / device time of the step,
          timed with CUDA events on the launching stream, inputs resident in HBM.
e2e     = the same bytes / wall time of the same step through the C ABI with pinned HOST buffers
          (kfr_dft_execute_batch_f32 with a NULL stream: H2D copy, kernels, D2H copy, synchronise).
roofline: the kernel with the largest share of the step (per-length CUDA-event timing), its algorithmic
          GB/s against MEASURED_PEAKS.json's HBM copy bandwidth.
cpu_baseline: KFR 7.0.1's own dft_plan<float> (compiled from the reference's sources on the host into
          oracle/_ref) on all host cores over a bounded sample of each batch, plus a one-core figure; the
          oracle's single-precision port where KFR was not built.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun each rank runs the full workload on its own GPU (batch sharding, no collective on the data
path; weak scaling); rank 0 prints one JSON line with the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIZES = [1000, 1536, 2187, 30720, 127, 8191]
BYTES_PER_SIZE = 256 << 20
METRIC = "batched c32 DFT GB/s (% of HBM roofline), chosen vs plain form at ≤1e-6 rel RMS"
FALLBACK_HBM_GBS = 6800.0

# DRAM bytes per signal measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum of one launch divided
# by the signals it processed; one-pass metrics captured on the full 256 MiB batches of this workload), from
# the k_c2c_pipe, k_fspt_cols / k_fspt_rows and k_rader_pfa launches summarised under profiles/.  Writes fall
# short of the algorithmic bytes by the output still in L2 when a launch ends.
NCU_TRAFFIC_BYTES_PER_SIGNAL: dict[int, float] = {
    1000: (268_458_240 + 221_152_000) / 33554,
    1536: (268_477_440 + 213_674_240) / 21845,
    2187: (268_476_672 + 216_896_512) / 15342,
    30720: (268_411_904 + 216_671_488 + 268_498_176 + 213_238_528) / 1092,
    127: (268_486_912 + 210_538_752) / 264208,
    8191: (268_598_272 + 214_211_072) / 4096,
}


def rel_rms(y, ref):
    """Relative RMS error of y against a reference."""
    y = np.asarray(y, dtype=np.complex128)
    ref = np.asarray(ref, dtype=np.complex128)
    return float(np.sqrt(np.sum(np.abs(y - ref) ** 2) / max(np.sum(np.abs(ref) ** 2), 1e-300)))


def batch_for(n: int) -> int:
    return BYTES_PER_SIZE // (8 * n)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join(tempfile.gettempdir(), f"kfr_gb300_clocks_gpu{gpu_index}_{os.getpid()}.csv")

    def start(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def count(self) -> int:
        """Samples written so far."""
        if self.proc is None:
            return 0
        try:
            self.f.flush()
            with open(self.path) as f:
                return sum(1 for line in f if line.count(",") >= 8)
        except OSError:
            return 0

    def keep_busy_until(self, samples: int, busy, limit_s: float = 3.0):
        """Runs busy() (one untimed step, synchronised) until `samples` samples exist or limit_s passes."""
        if self.proc is None:
            return
        t0 = time.perf_counter()
        while self.count() < samples and time.perf_counter() - t0 < limit_s:
            busy()

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(ngpus: int):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def make_inputs(torch, n, batch, seed, device):
    g = torch.Generator(device=device).manual_seed(seed)
    amp = 0.5 + float(np.random.default_rng(seed).uniform(0, 1))
    x = torch.randn(batch, n, dtype=torch.complex64, device=device, generator=g) * amp
    return x


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def cpu_baseline_run(frac: float = 1 / 32, threads: int | None = None, reps: int = 3) -> dict:
    """The reference's CPU path on the host cores over a bounded sample of each batch: KFR 7.0.1's own
    dft_plan<float> (oracle/_ref, compiled from the reference's sources on this machine), one plan per length
    built beforehand and shared by all threads, best of `reps` passes; where KFR was not built here, the
    oracle's single-precision port instead (kind "port").  Returns the cpu_baseline object."""
    from oracle.oracle import Oracle, available

    kind = "reference" if available("ref") else "port"
    orc = Oracle("ref" if kind == "reference" else "orc")
    threads = threads or os.cpu_count() or 1
    total_bytes, total_t = 0, 0.0
    for n in SIZES:
        b = max(1, int(batch_for(n) * frac))
        rng = np.random.default_rng(n)
        x = (rng.standard_normal((b, n)) + 1j * rng.standard_normal((b, n))).astype(np.complex64)
        if kind == "reference":
            dt = orc.dft_time(x, threads=threads, reps=reps)
        else:
            orc.dft(x[: max(1, b // 8)], precision="f32", threads=threads)  # warm the pages and plan path
            dt = 1e30
            for _ in range(reps):
                t0 = time.perf_counter()
                orc.dft(x, precision="f32", threads=threads)
                dt = min(dt, time.perf_counter() - t0)
        total_t += dt
        total_bytes += 16 * n * b
    what = ("KFR 7.0.1 dft_plan<float> compiled with g++ -O3 on this host" if kind == "reference" else
            "the oracle's single-precision port (KFR was not built on this host)")
    sample = (f"{what}; {frac:g} of each batch ({BYTES_PER_SIZE * frac / 2**20:g} MiB per length), forward, "
              f"{threads} thread(s), plan built once, best of {reps}")
    return {"value": round(total_bytes / total_t / 1e9, 3), "unit": "GB/s", "cores": threads, "kind": kind,
            "sample": sample, "cpu": cpu_model()}


def cpu_baseline_both() -> dict:
    """All host cores (the cpu_baseline value) plus a one-core figure on a smaller sample."""
    allc = cpu_baseline_run(1 / 32)
    one = cpu_baseline_run(1 / 256, threads=1)
    allc["one_core"] = {"value": one["value"], "sample": one["sample"]}
    return allc


def measure_rows(torch, k, dev, stream, hbm, with_cpu):
    """The other rows of the DFT path on their own configurations (device-resident inputs, CUDA events,
    L2 flushed between repetitions where the data would fit in it), each beside the oracle's single-precision
    port on a bounded sample on all host cores."""
    from oracle.oracle import Oracle

    orc = Oracle("orc") if with_cpu else None
    threads = os.cpu_count() or 1
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def timed(fn, reps=5, flush_l2=False):
        fn()
        torch.cuda.synchronize()
        tot = 0.0
        for _ in range(reps):
            if flush_l2:
                flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / reps

    def cpu(fn, nbytes):
        if orc is None:
            return None
        fn()  # warm
        t0 = time.perf_counter()
        fn()
        return round(nbytes / (time.perf_counter() - t0) / 1e9, 3)

    rows = {}
    g = torch.Generator(device=dev).manual_seed(77)
    # real DFT f32, N in {1920, 44100, 48000}, 256 MiB of reals each, CCs
    for n in (1920, 44100, 48000):
        b = (256 << 20) // (4 * n)
        plan = k.dft_plan_real(n)
        x = torch.randn(b, n, device=dev, generator=g)
        y = torch.empty(b, n // 2 + 1, dtype=torch.complex64, device=dev)
        ms = timed(lambda: plan.execute_batch(y, x, b, stream=stream))
        nb = b * (4 * n + 8 * (n // 2 + 1))
        xs = x[: max(1, b // 64)].cpu().numpy()
        rows[f"real_dft_{n}"] = {
            "batch": b, "ms": round(ms, 4), "gbs": round(nb / (ms * 1e-3) / 1e9, 1),
            "frac": round(nb / (ms * 1e-3) / 1e9 / hbm, 4),
            "cpu_port_gbs": cpu(lambda: orc.dft_real(xs, precision="f32", threads=threads),
                                len(xs) * (4 * n + 8 * (n // 2 + 1)))}
        if n == 1920:
            # the inverse (CCs spectrum -> reals) on the same batch
            ms_i = timed(lambda: plan.execute_batch(x, y, b, inverse=True, stream=stream))
            rows[f"real_dft_inverse_{n}"] = {"batch": b, "ms": round(ms_i, 4), "gbs": round(nb / (ms_i * 1e-3) / 1e9, 1),
                                             "frac": round(nb / (ms_i * 1e-3) / 1e9 / hbm, 4)}
        del x, y, plan
    # DCT-II of 4096 x 512 (16 MiB: L2 flushed between repetitions)
    b, n = 4096, 512
    plan = k.dct_plan(n)
    x = torch.rand(b, n, device=dev, generator=g) * 2 - 1
    y = torch.empty_like(x)
    ms = timed(lambda: plan.execute_batch(y, x, b, stream=stream), flush_l2=True)
    # the same call issued back to back on 16 distinct input / output pairs (256 MiB, more than L2): the
    # device rate once the per-call host cost overlaps earlier calls
    xs16 = [torch.rand(b, n, device=dev, generator=g) * 2 - 1 for _ in range(16)]
    ys16 = [torch.empty_like(x) for _ in range(16)]

    def dct16():
        for xi, yi in zip(xs16, ys16):
            plan.execute_batch(yi, xi, b, stream=stream)

    ms16 = timed(dct16, reps=3) / 16
    xs = x[:1024].cpu().numpy()
    rows["dct2_4096x512"] = {"ms": round(ms, 4), "gbs": round(8 * n * b / (ms * 1e-3) / 1e9, 1),
                             "frac": round(8 * n * b / (ms * 1e-3) / 1e9 / hbm, 4),
                             "ms_back_to_back": round(ms16, 4),
                             "gbs_back_to_back": round(8 * n * b / (ms16 * 1e-3) / 1e9, 1),
                             "frac_back_to_back": round(8 * n * b / (ms16 * 1e-3) / 1e9 / hbm, 4),
                             "cpu_port_gbs": cpu(lambda: orc.dct(xs, precision="f32", threads=threads), 8 * n * 1024)}
    del x, y, plan, xs16, ys16
    # convolution filter: 64 signals of 2^20 f32, 1023 taps, block 1024 (each signal from a reset state)
    chans, L, M = 64, 1 << 20, 1023
    taps = torch.randn(M, device=dev, generator=g) / M
    f = k.convolve_filter(taps, 1024, dtype="f32", channels=chans)
    x = torch.randn(chans, L, device=dev, generator=g)
    y = torch.empty_like(x)

    def run_filter():
        f.reset()
        f.apply(y, x)

    ms = timed(run_filter, reps=3)
    nb = chans * 8 * L + 4 * M
    xs = x[0].cpu().numpy()
    hs = taps.cpu().numpy()

    def cpu_filter():
        flt = orc.filter(hs, 1024, precision="f32")
        flt.process(xs)

    rows["convolve_filter_64x2^20_1023taps"] = {
        "ms": round(ms, 3), "gbs": round(nb / (ms * 1e-3) / 1e9, 1), "frac": round(nb / (ms * 1e-3) / 1e9 / hbm, 4),
        "cpu_port_gbs": cpu(cpu_filter, 8 * L), "cpu_sample": "one 2^20 signal, one core (streaming filter)"}
    del x, y, f
    # large single transforms: c32 2^24 and 30,720,000, c64 2^20
    for n, dt, name in ((1 << 24, torch.complex64, "c32_2^24"), (30720000, torch.complex64, "c32_30720000"),
                        (1 << 20, torch.complex128, "c64_2^20")):
        sfx = "f32" if dt == torch.complex64 else "f64"
        plan = k.dft_plan(n, sfx)
        x = torch.randn(n, dtype=dt, device=dev, generator=g)
        y = torch.empty_like(x)
        tmp = torch.empty(max(1, plan.temp_size_batch(1)), dtype=torch.uint8, device=dev)
        ms = timed(lambda: plan.execute_batch(y, x, 1, temp=tmp, stream=stream), flush_l2=n * 16 < (256 << 20))
        nb = (16 if sfx == "f32" else 32) * n
        rows[name] = {"ms": round(ms, 4), "gbs": round(nb / (ms * 1e-3) / 1e9, 1),
                      "frac": round(nb / (ms * 1e-3) / 1e9 / hbm, 4), "plan": plan.describe()}
        if name == "c32_2^24" and orc is not None:
            xs = x.cpu().numpy().reshape(1, n)
            rows[name]["cpu_port_gbs"] = cpu(lambda: orc.dft(xs, precision="f32", threads=threads), nb)
        del x, y, tmp, plan
    # power-of-two lengths 2^10 .. 2^24, 1 GiB batches
    pw = {}
    for e in (10, 12, 14, 16, 18, 20, 22, 24):
        n = 1 << e
        b = (1 << 30) // (8 * n)
        plan = k.dft_plan(n)
        x = torch.randn(b, n, dtype=torch.complex64, device=dev, generator=g)
        y = torch.empty_like(x)
        tmp = torch.empty(max(1, plan.temp_size_batch(b)), dtype=torch.uint8, device=dev)
        ms = timed(lambda: plan.execute_batch(y, x, b, temp=tmp, stream=stream), reps=3)
        gbs = 16 * n * b / (ms * 1e-3) / 1e9
        pw[f"2^{e}"] = {"batch": b, "ms": round(ms, 4), "gbs": round(gbs, 1), "frac": round(gbs / hbm, 4),
                        "plan": plan.describe()[:60]}
        del x, y, tmp, plan
    rows["pow2_c32_1GiB"] = pw
    # the precision configuration: c32 at N = 2^12, 2^16, 2^20, 2^24 with 1 GiB batches, the FP32 CUDA-core plan
    # beside the tensor-core radix-16 plans (FP16 hi + lo scaled per butterfly; BF16 hi + mid + lo); errors on
    # the precision workload (sum of 64 random sinusoids + 1e-3 noise) against numpy's FP64 FFT
    from kfr_gb300.workloads import precision_signals

    prec = {}
    for e, nerr in ((12, 8), (16, 4), (20, 2), (24, 1)):
        n = 1 << e
        b = (1 << 30) // (8 * n)
        X = torch.randn(b, n, dtype=torch.complex64, device=dev, generator=g)
        Y = torch.empty_like(X)
        xs = precision_signals(n, nerr, 4000 + e)
        ref = np.fft.fft(xs.astype(np.complex128), axis=-1)
        xd = torch.from_numpy(xs).to(dev)
        yd = torch.empty_like(xd)
        row = {"batch": b}
        for name, plan in (("fp32_cuda_cores", k.dft_plan(n)), ("tensor_fp16x2_scaled", k.dft_plan_tensor(n, "fp16")),
                           ("tensor_bf16x3", k.dft_plan_tensor(n, "bf16"))):
            tmp = torch.empty(max(1, plan.temp_size_batch(b)), dtype=torch.uint8, device=dev)
            ms = timed(lambda: plan.execute_batch(Y, X, b, temp=tmp, stream=stream), reps=3)
            plan.execute_batch(yd, xd, nerr, temp=tmp)
            y = yd.cpu().numpy()
            gbs = 16 * n * b / (ms * 1e-3) / 1e9
            row[name] = {"ms": round(ms, 4), "gbs": round(gbs, 1), "frac": round(gbs / hbm, 4),
                         "rel_rms": float(f"{rel_rms(y, ref):.3e}"),
                         "max_rel": float(f"{np.max(np.abs(y - ref)) / np.max(np.abs(ref)):.3e}"),
                         "plan": plan.describe()[:90]}
            del tmp, plan
        prec[f"2^{e}"] = row
        del X, Y, xd, yd
    rows["precision_c32_1GiB"] = prec
    del flush
    return rows


def run_reference(args):
    rank, world, local = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")), 0
    if rank != 0:
        return 0
    for _ in range(args.warmup):
        cpu_baseline_run(1 / 128, reps=1)
    vals = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        cb = cpu_baseline_run(1 / 32, reps=1)
        vals.append(cb["value"])
    wall = time.perf_counter() - t0
    value = float(np.mean(vals))
    cb["value"] = round(value, 3)
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(wall / args.steps * 1e3, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config_dict(),
        "cpu_baseline": cb,
        "e2e": {"value": round(value, 3), "unit": "GB/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def run_case(spec: str) -> int:
    """One plan on device-resident c32 signals, three executions, for a profiler to capture: form "plain"
    (the default plan) or "fp16" / "bf16" (the tensor-core plans), length n, `MiB` of signals (default 128)."""
    import torch

    import kfr_gb300 as k

    parts = spec.split(":")
    if parts[0] == "uneven":
        # the uneven batch: `n` signals of log-uniform lengths on [64, 65536] in one persistent launch
        from kfr_gb300.workloads import uneven_lengths

        lengths = uneven_lengths(int(parts[1]))
        up = k.dft_plan_uneven(lengths, autotune=not (len(parts) > 2 and parts[2] == "fixed"))
        x = torch.randn(int(sum(lengths)), dtype=torch.complex64, device="cuda")
        y = torch.empty_like(x)
        for _ in range(3):
            up.execute(y, x)
        torch.cuda.synchronize()
        print(json.dumps({"case": spec, "elements": int(sum(lengths)), "plan": up.describe()}))
        return 0
    if parts[0] == "dct":
        # DCT-II of `MiB` of f32 signals of length n, three calls back to back on a stream
        n = int(parts[1])
        mib = int(parts[2]) if len(parts) > 2 else 16
        b = max(1, (mib << 20) // (4 * n))
        plan = k.dct_plan(n)
        x = torch.rand(b, n, device="cuda") * 2 - 1
        y = torch.empty_like(x)
        st = torch.cuda.Stream()
        for _ in range(3):
            plan.execute_batch(y, x, b, stream=st.cuda_stream)
        torch.cuda.synchronize()
        print(json.dumps({"case": spec, "batch": b}))
        return 0
    if parts[0] == "real":
        # the forward real DFT (CCs) of `MiB` of f32 signals of length n
        n = int(parts[1])
        mib = int(parts[2]) if len(parts) > 2 else 128
        b = max(1, (mib << 20) // (4 * n))
        plan = k.dft_plan_real(n)
        x = torch.randn(b, n, device="cuda")
        y = torch.empty(b, n // 2 + 1, dtype=torch.complex64, device="cuda")
        for _ in range(3):
            plan.execute_batch(y, x, b)
        torch.cuda.synchronize()
        print(json.dumps({"case": spec, "batch": b}))
        return 0
    form, n = parts[0], int(parts[1])
    mib = int(parts[2]) if len(parts) > 2 else 128
    b = max(1, (mib << 20) // (8 * n))
    plan = k.dft_plan(n) if form == "plain" else k.dft_plan_tensor(n, form)
    x = torch.randn(b, n, dtype=torch.complex64, device="cuda")
    y = torch.empty_like(x)
    tmp = torch.empty(max(1, plan.temp_size_batch(b)), dtype=torch.uint8, device="cuda")
    for _ in range(3):
        plan.execute_batch(y, x, b, temp=tmp)
    torch.cuda.synchronize()
    print(json.dumps({"case": spec, "batch": b, "plan": plan.describe()}))
    return 0


def config_dict():
    return {"workload": "c32 forward DFT, N in {1000,1536,2187,30720,127,8191}, 256 MiB batch per N",
            "sizes": SIZES, "batches": [batch_for(n) for n in SIZES], "bytes_per_n": BYTES_PER_SIZE,
            "l2": "every input (256 MiB) exceeds L2; no flush needed", "form": "plain"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-uneven", action="store_true", help="skip the uneven-batch comparison")
    ap.add_argument("--no-rows", action="store_true", help="skip the real / DCT / filter / large-single rows")
    ap.add_argument("--sizes", type=str, default=None, help="comma-separated subset of the lengths (profiling)")
    ap.add_argument("--batch-mib", type=int, default=None, help="MiB per length instead of 256 (profiling)")
    ap.add_argument("--case", type=str, default=None,
                    help="profiling: run one plan `form:n[:MiB]` three times and exit (form: plain, fp16, bf16, "
                         "real, dct; or uneven:count[:fixed], fixed = no autotuning)")
    args = ap.parse_args()
    if args.case:
        return run_case(args.case)
    global SIZES, BYTES_PER_SIZE
    if args.sizes:
        SIZES = [int(v) for v in args.sizes.split(",")]
    if args.batch_mib:
        BYTES_PER_SIZE = args.batch_mib << 20
    if args.impl == "reference":
        return run_reference(args)

    import torch

    import kfr_gb300 as k

    rank, world, local = dist_setup(args.gpus)
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    # a stream of our own: the C ABI runs calls on a NULL stream (the default stream's handle) synchronously,
    # and the timed steps are stream-ordered enqueues
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)
    hbm, peak_kind = peaks()

    plans, xs, ys = {}, {}, {}
    for i, n in enumerate(SIZES):
        plans[n] = k.dft_plan(n, "f32")
        xs[n] = make_inputs(torch, n, batch_for(n), 1000 + i + 97 * rank, dev)
        ys[n] = torch.empty_like(xs[n])
    temps = {n: torch.empty(max(1, plans[n].temp_size_batch(batch_for(n))), dtype=torch.uint8, device=dev)
             for n in SIZES}

    def step(events=None):
        for n in SIZES:
            if events is not None:
                events[n][0].record(stream)
            plans[n].execute_batch(ys[n], xs[n], batch_for(n), temp=temps[n], stream=stream)
            if events is not None:
                events[n][1].record(stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()

    # accuracy on a sample of each batch (outside the timed region), against numpy's FP64 FFT (same sign and
    # scaling convention: forward e^{-2 pi i n k / N}, unscaled)
    errs = {}
    for n in SIZES:
        s = min(8, batch_for(n))
        ref = np.fft.fft(xs[n][:s].cpu().numpy().astype(np.complex128), axis=-1)
        errs[n] = rel_rms(ys[n][:s].cpu().numpy(), ref)

    clocks = ClockSampler(local)
    ev = {n: [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)] for n in SIZES}
    start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    def busy_step():
        step()
        torch.cuda.synchronize()

    # The timed region (~1 ms per step) is shorter than nvidia-smi's 200 ms sampling period, so the sampler
    # runs over a loaded window: untimed steps of the same workload until its first sample, the timed
    # region, then untimed steps until one more sample lands after it.
    clocks.start()
    clocks.keep_busy_until(1, busy_step)
    barrier(world)
    torch.cuda.synchronize()
    start.record(stream)
    for s in range(args.steps):
        step({n: ev[n][s] for n in SIZES})
    stop.record(stream)
    torch.cuda.synchronize()
    clocks.keep_busy_until(clocks.count() + 1, busy_step)
    clk = clocks.stop()
    clk["window"] = "untimed steps of the same workload around the timed region (sampling period 200 ms)"
    barrier(world)
    total_ms = max_over_ranks(start.elapsed_time(stop), world)
    ms_step = total_ms / args.steps
    bytes_step = sum(16 * n * batch_for(n) for n in SIZES)
    value = bytes_step * world / (ms_step * 1e-3) / 1e9

    per = {}
    for n in SIZES:
        ms = float(np.mean([a.elapsed_time(b) for a, b in ev[n]]))
        gbs = 16 * n * batch_for(n) / (ms * 1e-3) / 1e9
        per[n] = {"ms": round(ms, 4), "gbs": round(gbs, 1), "frac": round(gbs / hbm, 4),
                  "gflops": round(5 * n * np.log2(n) * batch_for(n) / (ms * 1e-3) / 1e9, 1),
                  "rel_rms": float(f"{errs[n]:.3e}"), "plan": plans[n].describe()}
    dom = max(SIZES, key=lambda n: per[n]["ms"])
    traffic = NCU_TRAFFIC_BYTES_PER_SIGNAL.get(dom)
    roof = {"bound": "hbm", "achieved": per[dom]["gbs"], "peak": hbm, "unit": "GB/s",
            "frac": per[dom]["frac"], "traffic": (traffic * batch_for(dom)) if traffic else None,
            "kernel": f"N={dom}: {plans[dom].describe()}", "peak_kind": peak_kind,
            "step_frac": round(value / world / hbm, 4)}
    launches = args.steps * sum(plans[n].launch_count(batch_for(n)) for n in SIZES)

    # end to end through the C ABI with pinned host buffers
    e2e = None
    if not args.no_e2e:
        hin = {n: xs[n].cpu().pin_memory() for n in SIZES}
        hout = {n: torch.empty_like(hin[n]).pin_memory() for n in SIZES}

        def e2e_step():
            for n in SIZES:
                plans[n].execute_batch(hout[n], hin[n], batch_for(n))

        for _ in range(max(1, args.warmup)):
            e2e_step()
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(args.steps):
            e2e_step()
        wall = max_over_ranks(time.perf_counter() - t0, world)
        e2e = {"value": round(bytes_step * world / (wall / args.steps) / 1e9, 3), "unit": "GB/s",
               "h2d_bytes_per_step": bytes_step // 2, "d2h_bytes_per_step": bytes_step // 2,
               "ms_per_step": round(wall / args.steps * 1e3, 3)}
        del hin, hout

    # uneven batch: 8192 signals of log-uniform lengths on [64, 65536] (7-smooth, 10% prime) in one
    # persistent launch (graph-replayed) against one plain plan execution per signal
    uneven = None
    if rank == 0 and not args.no_uneven and not args.sizes:
        from kfr_gb300.workloads import uneven_lengths

        lengths = uneven_lengths(8192)
        up = k.dft_plan_uneven(lengths, autotune=True)
        total = int(sum(lengths))
        g = torch.Generator(device=dev).manual_seed(4242)
        ux = torch.complex(torch.rand(total, device=dev, generator=g) * 2 - 1,
                           torch.rand(total, device=dev, generator=g) * 2 - 1)
        uy = torch.empty_like(ux)

        def timed(fn, reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            for _ in range(reps):
                fn()
            e1.record(stream)
            torch.cuda.synchronize()
            return e0.elapsed_time(e1) / reps

        for _ in range(3):
            up.execute(uy, ux, stream=stream)
        ms_p = timed(lambda: up.execute(uy, ux, stream=stream), 10)
        up.execute_per_signal(uy, ux, stream=stream)
        ms_s = timed(lambda: up.execute_per_signal(uy, ux, stream=stream), 2)
        # the batched plain form: the signals of each length stored contiguously (as if the caller had sorted
        # them by length) and one batched plan execution per distinct length
        classes = {}
        for n in lengths:
            classes[n] = classes.get(n, 0) + 1
        cplans, cbufs = [], []
        for n, c in sorted(classes.items()):
            pl = k.dft_plan(n)
            xb = torch.randn(c, n, dtype=torch.complex64, device=dev, generator=g)
            tb = torch.empty(max(1, pl.temp_size_batch(c)), dtype=torch.uint8, device=dev)
            cplans.append((pl, c))
            cbufs.append((xb, torch.empty_like(xb), tb))

        def per_class():
            for (pl, c), (xb, yb, tb) in zip(cplans, cbufs):
                pl.execute_batch(yb, xb, c, temp=tb, stream=stream)

        per_class()
        ms_c = timed(per_class, 3)
        del cplans, cbufs
        ub = 16 * total
        uneven = {"signals": len(lengths), "elements": total, "persistent_ms": round(ms_p, 4),
                  "persistent_gbs": round(ub / (ms_p * 1e-3) / 1e9, 1), "per_signal_ms": round(ms_s, 3),
                  "per_signal_gbs": round(ub / (ms_s * 1e-3) / 1e9, 1), "speedup": round(ms_s / ms_p, 2),
                  "length_classes": len(classes), "per_class_batched_ms": round(ms_c, 4),
                  "per_class_batched_gbs": round(ub / (ms_c * 1e-3) / 1e9, 1),
                  "frac": round(ub / (ms_p * 1e-3) / 1e9 / hbm, 4),
                  "plan": up.describe()}
        del ux, uy, up

    rows = None
    if rank == 0 and not args.no_rows and not args.sizes:
        rows = measure_rows(torch, k, dev, stream, hbm, not args.no_cpu)

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = cpu_baseline_both()

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "GB/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_step, 4), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded N(0,1) x amplitude, c32",
            "config": config_dict(), "roofline": roof, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clk, "per_size": {str(n): per[n] for n in SIZES}, "uneven": uneven,
            "rows": rows,
            "max_rel_rms": float(f"{max(errs.values()):.3e}"),
        }
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())

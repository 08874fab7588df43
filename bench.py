#!/usr/bin/env python
"""Benchmark: JTransforms' transform path on GB300.

Headline workload (one JSON line): FloatFFT_1D.complexForward batched at
n = 2^10, 2^14, 2^18, 2^20, 2^24, each a 1 GiB complex64 array
(batch = 2^27 / n), inputs i.i.d. N(0,1) re/im from a seeded generator.
A step runs the five 1 GiB batches once.  GFLOP/s uses 5 N log2 N per
transform.  The other workloads (256 x DoubleFFT_1D(4096) forward+inverse,
FloatFFT_2D(2048^2).realForward, DoubleDCT_2D(1024^2).forward(true),
DoubleFFT_3D(256^3).complexForward, DoubleDST_3D/DoubleDHT_3D(128^3).forward,
10,000 mixed 1D transforms) are reported under "other_workloads".

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference (oracle/, no JDK
on the box to run JTransforms itself) on all host cores for the same
workload, on a bounded sample of each batch.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIZES = [2 ** 10, 2 ** 14, 2 ** 18, 2 ** 20, 2 ** 24]
HEADLINE_SIZES = list(SIZES)
# DRAM bytes (read + write) of one headline step, from an ncu capture
# (dram__bytes_read.sum + dram__bytes_write.sum, L2 kept between launches) of
# the 256 MiB-per-size case, scaled by 4 (traffic grows with the transforms
# processed): 2144 + 2142 + 3827 + 3789 + 6310 MB for 2^10 .. 2^24 (one pass,
# one, two, two, three: each pass reads and writes the array)
TRAFFIC_PER_STEP = 18.21e9
ELEMS = 2 ** 27          # complex elements per size per rank (1 GiB complex64)
SEED = 20110602
METRIC = "GFLOP/s (5N log2N) & % HBM roofline; TC-split vs plain FP32 at same error"
UNIT = "GFLOP/s"
L2_FLUSH_BYTES = 256 << 20


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d.get("hbm_gbs", 6800.0)), "measured"
    return 6800.0, "fallback"


def flops_c2c(n, batch):
    return 5.0 * n * math.log2(n) * batch


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 50 ms, each line
    time-stamped on arrival; summary() keeps the samples inside a window."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self, t0=None, t1=None):
        """Median SM clock and the throttle reasons seen in [t0, t1], plus the
        last sample before t0 and the first after t1 (the clock state that
        the window starts and ends in)."""
        rows = list(self.lines)
        if t0 is not None:
            inside = [r for r in rows if t0 <= r[0] <= t1]
            before = [r for r in rows if r[0] < t0][-1:]
            after = [r for r in rows if r[0] > t1][:1]
            rows = before + inside + after
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, ln in rows:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() in ("active", "1", "yes"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# Replicas: every rank transforms its own batch (weak scaling); the only
# cross-rank traffic is the start barrier and the max of the step times.
def dist_init(world: int, backend: str = "nccl"):
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group(backend)


def dist_barrier(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def dist_finish(world: int):
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


# ----------------------------------------------------------------------------
# reference arm: the oracle (CPU restatement of JTransforms) on host cores
# ----------------------------------------------------------------------------
def cpu_sample(budget_s: float = 3.0, threads: int = 0):
    """Times the oracle on a bounded sample of each headline batch.  Returns
    (GFLOP/s, threads, description)."""
    from oracle import oracle as O
    O.build()
    nthreads = threads or O.max_threads()
    rng = np.random.default_rng(SEED)
    tot_flops, tot_time, parts = 0.0, 0.0, []
    for n in SIZES:
        batch = ELEMS // n
        x1 = rng.standard_normal(2 * n).astype(np.float32)
        t0 = time.perf_counter()
        O.run(O.FFT, O.COMPLEX_FORWARD, [n], x1)
        t1 = time.perf_counter() - t0
        per_thread = max(1, int(budget_s / max(t1, 1e-6)))
        count = int(min(batch, max(1, per_thread * nthreads)))
        x = rng.standard_normal(2 * n * count).astype(np.float32)
        t0 = time.perf_counter()
        O.run_batch(O.FFT, O.COMPLEX_FORWARD, [n], x, count, 2 * n, False, nthreads)
        dt = time.perf_counter() - t0
        tot_flops += flops_c2c(n, count)
        tot_time += dt
        parts.append(f"2^{int(math.log2(n))}x{count}")
    return tot_flops / tot_time / 1e9, nthreads, "oracle complexForward on " + ", ".join(parts) + " of the 1 GiB batches"


def run_reference(args, world, rank):
    if rank != 0:
        return 0
    vals = []
    kind = "port"
    threads = 0
    desc = ""
    for _ in range(args.warmup):
        cpu_sample(0.3)
    for _ in range(args.steps):
        v, threads, desc = cpu_sample(1.0)
        vals.append(v)
    value = statistics.median(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded N(0,1))",
            "config": headline_config(args),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind, "sample": desc},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "JTransforms is Java and no JDK exists on the box; the reference arm runs oracle/jt_oracle.cpp, "
                    "a C++ restatement of its algorithms, with OpenMP across the batch"}
    print(json.dumps(line), flush=True)
    return 0


def headline_config(args):
    return {"workload": "FloatFFT_1D.complexForward batched, n=2^10,2^14,2^18,2^20,2^24, 1 GiB complex64 each "
                        "(batch=2^27/n), inputs N(0,1)",
            "sizes": SIZES, "elems_per_size": ELEMS, "global_batch": [ELEMS // n for n in SIZES],
            "parallelism": f"replicas{args.gpus}",
            "l2": "inputs 1 GiB > L2; a 256 MiB buffer is also written before each timed call",
            "mode": "plain FP32 CUDA cores", "tma_pipeline": not getattr(args, "no_tma", False)}


# ----------------------------------------------------------------------------
# our arm
# ----------------------------------------------------------------------------
def timed_calls(fn_list, restore, flush, steps, warmup, stream):
    """Runs each fn once per step bracketed by CUDA events on `stream`; restore
    and flush run outside the events.  Returns per-fn lists of ms."""
    import torch
    times = [[] for _ in fn_list]
    for s in range(warmup + steps):
        for i, fn in enumerate(fn_list):
            restore(i)
            flush()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            if s >= warmup:
                times[i].append((e0, e1))
    torch.cuda.synchronize()
    return [[a.elapsed_time(b) for a, b in t] for t in times]


def link_bandwidth(host_np, dev):
    """Host<->device copy bandwidth of a 1 GiB pinned array (GB/s): one
    direction at a time, and both at once on two streams (the bound of the
    end-to-end leg, whose copies in and out overlap)."""
    import torch
    h = torch.from_numpy(host_np)
    d = torch.empty_like(dev)
    d2 = torch.empty_like(dev)
    h2 = torch.empty(h.numel(), dtype=h.dtype, pin_memory=True)
    nbytes = h.numel() * h.element_size()
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    out = {}
    for name in ("h2d", "d2h", "bidirectional"):
        best = 1e9
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if name in ("h2d", "bidirectional"):
                with torch.cuda.stream(s1):
                    d.copy_(h, non_blocking=True)
            if name in ("d2h", "bidirectional"):
                with torch.cuda.stream(s2):
                    h2.copy_(d2, non_blocking=True)
            torch.cuda.synchronize()
            best = min(best, time.perf_counter() - t0)
        out[name] = (2 if name == "bidirectional" else 1) * nbytes / best / 1e9
    return out


def sixty_db(n, gen):
    """Input set (b), 60 dB dynamic range: 8 unit-amplitude complex
    exponentials at random bins (random phases) plus 1e-3 N(0,1), as
    interleaved complex64 on the device."""
    import torch
    j = torch.arange(n, device="cuda", dtype=torch.int64)
    bins = torch.randint(0, n, (8,), device="cuda", generator=gen)
    ph = torch.rand(8, device="cuda", dtype=torch.float64, generator=gen) * 2 * math.pi
    ang = 2 * math.pi * ((j[:, None] * bins[None, :]) % n).double() / n + ph[None, :]
    z = torch.polar(torch.ones_like(ang), ang).sum(1)
    z = z + 1e-3 * torch.complex(torch.randn(n, device="cuda", dtype=torch.float64, generator=gen),
                                 torch.randn(n, device="cuda", dtype=torch.float64, generator=gen))
    return torch.view_as_real(z.to(torch.complex64)).reshape(-1).contiguous()


def blob_image(size, rng):
    """Sum of 20 Gaussian blobs (centres U[0,size)^2, sigma U[5,50] px,
    amplitude U[0,1]) plus N(0, 0.01^2) noise."""
    yy, xx = np.mgrid[0:size, 0:size].astype(np.float64)
    img = np.zeros((size, size))
    for _ in range(20):
        cy, cx = rng.uniform(0, size, 2)
        s = rng.uniform(5, 50)
        a = rng.uniform(0, 1)
        img += a * np.exp(-((yy - cy) ** 2 + (xx - cx) ** 2) / (2 * s * s))
    img += rng.normal(0, 0.01, img.shape)
    return img


def other_workloads(args, peak, flush, stream):
    import torch
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    out = {}
    rng = np.random.default_rng(SEED)
    # median and best of at least 20 runs after the warm-up
    steps, warm = max(args.steps, 20), args.warmup
    # compute rooflines: CUDA-core FMA throughput measured on this GPU
    fma = {}
    for key, prec in (("fp64", N.FLOAT64), ("fp32", N.FLOAT32)):
        v = ctypes.c_double()
        if N.load().jt_fma_peak(prec, ctypes.byref(v)) == N.OK:
            fma[key] = v.value
    out["fma_peak_GFLOPs"] = fma

    def bound(entry, flops, bytes_alg, ms, prec):
        # the roofline of a Double (or Float) workload: min(HBM x intensity,
        # CUDA-core FMA peak) on the convention's flop count
        cpeak = fma.get(prec)
        gf = flops / (ms * 1e-3) / 1e9
        hbm_lim = peak * flops / bytes_alg
        entry["hbm_frac"] = (bytes_alg / (ms * 1e-3) / 1e9) / peak
        if cpeak:
            entry[f"{prec}_frac_nominal"] = gf / cpeak
            entry["attainable_GFLOP/s"] = min(hbm_lim, cpeak)
            entry["binding"] = prec if cpeak < hbm_lim else "hbm"
            entry["frac_of_attainable"] = gf / min(hbm_lim, cpeak)

    def errors(entry, got, want):
        # relative L2 and max error (max |got - want| / max |want|) of the
        # last timed call's output against an FP64 reference
        g64 = np.asarray(got, dtype=np.float64).ravel()
        w64 = np.asarray(want, dtype=np.float64).ravel()
        d = g64 - w64
        entry["rel_l2_vs_fp64"] = float(np.linalg.norm(d) / np.linalg.norm(w64))
        entry["rel_max_err_vs_fp64"] = float(np.abs(d).max() / np.abs(w64).max())

    def measure(name, plan, op, buf, batch, dist, scale, flops, bytes_alg, unit_note, ref_fn=None):
        pristine = buf.clone()
        fns = [lambda: plan.execute(op, buf, 0, scale, batch=batch, dist=dist)]
        t = timed_calls(fns, lambda i: buf.copy_(pristine), flush, steps, warm, stream)[0]
        ms = statistics.median(t)
        out[name] = {"value": flops / (ms * 1e-3) / 1e9, "unit": "GFLOP/s", "ms": ms, "best_ms": min(t),
                     "flops": unit_note}
        bound(out[name], flops, bytes_alg, ms, "fp64" if buf.dtype == torch.float64 else "fp32")
        if ref_fn is not None:  # buf holds the last timed call's output
            errors(out[name], buf.cpu().numpy(), ref_fn(pristine.cpu().numpy()))

    # config 1: 256 x DoubleFFT_1D(4096) complexForward then complexInverse(scale=true)
    n, B = 4096, 256
    f1 = J.DoubleFFT_1D(n)
    buf = torch.from_numpy(rng.uniform(-1, 1, 2 * n * B)).cuda()
    pristine = buf.clone()

    def fwd_inv():
        f1.plan.execute(N.COMPLEX_FORWARD, buf, 0, False, batch=B, dist=2 * n)
        f1.plan.execute(N.COMPLEX_INVERSE, buf, 0, True, batch=B, dist=2 * n)
    t = timed_calls([fwd_inv], lambda i: buf.copy_(pristine), flush, steps, warm, stream)[0]
    ms = statistics.median(t)
    out["c1_DoubleFFT_1D_4096x256_fwd_inv"] = {
        "value": 2 * flops_c2c(n, B) / (ms * 1e-3) / 1e9, "unit": "GFLOP/s", "ms": ms,
        "flops": "5N log2N x2 directions"}
    bound(out["c1_DoubleFFT_1D_4096x256_fwd_inv"], 2 * flops_c2c(n, B), 4 * 16 * n * B, ms, "fp64")
    # the forward half against torch's complex128 FFT of the same arrays
    y = pristine.clone()
    f1.plan.execute(N.COMPLEX_FORWARD, y, 0, False, batch=B, dist=2 * n)
    z = torch.fft.fft(torch.view_as_complex(pristine.view(B, n, 2)), dim=1)
    errors(out["c1_DoubleFFT_1D_4096x256_fwd_inv"], y.cpu().numpy(), torch.view_as_real(z).cpu().numpy())

    # config 2a: FloatFFT_2D(2048, 2048).realForward on a blob image
    img = blob_image(2048, rng).astype(np.float32).ravel()
    f2 = J.FloatFFT_2D(2048, 2048)
    buf = torch.from_numpy(img).cuda()
    N2 = 2048 * 2048
    def packed2d(a, R=2048, C=2048):
        # numpy's FP64 spectrum in realForward's packed 2D layout
        # (fft/DoubleFFT_2D.java:788-815)
        F = np.fft.rfft2(a.astype(np.float64).reshape(R, C))
        P = np.empty((R, C))
        P[:, 2::2] = F[:, 1:C // 2].real
        P[:, 3::2] = F[:, 1:C // 2].imag
        k = np.arange(1, R // 2)
        P[k, 0] = F[k, 0].real
        P[k, 1] = F[k, 0].imag
        P[R - k, 1] = F[k, C // 2].real
        P[R - k, 0] = -F[k, C // 2].imag
        P[0, 0], P[0, 1] = F[0, 0].real, F[0, C // 2].real
        P[R // 2, 0], P[R // 2, 1] = F[R // 2, 0].real, F[R // 2, C // 2].real
        return P
    measure("c2a_FloatFFT_2D_2048_realForward", f2.plan, N.REAL_FORWARD, buf, 1, N2, False,
            2.5 * N2 * math.log2(N2), 2 * 4 * N2, "2.5N log2N", ref_fn=packed2d)
    # config 2b: DoubleDCT_2D(1024, 1024).forward(scale=true)
    img = blob_image(1024, rng).ravel()
    d2 = J.DoubleDCT_2D(1024, 1024)
    buf = torch.from_numpy(img).cuda()
    N2 = 1024 * 1024
    import scipy.fft as sfft
    measure("c2b_DoubleDCT_2D_1024_forward", d2.plan, N.FORWARD, buf, 1, N2, True,
            2.5 * N2 * math.log2(N2), 2 * 8 * N2, "2.5N log2N",
            ref_fn=lambda a: sfft.dctn(a.reshape(1024, 1024), type=2, norm="ortho"))
    # config 3a: DoubleFFT_3D(256^3).complexForward, N(0,1)
    f3 = J.DoubleFFT_3D(256, 256, 256)
    N3 = 256 ** 3
    g = torch.Generator(device="cuda").manual_seed(SEED)
    buf = torch.randn(2 * N3, dtype=torch.float64, device="cuda", generator=g)
    def fft3(a):
        z = np.fft.fftn((a[0::2] + 1j * a[1::2]).reshape(256, 256, 256))
        r = np.empty(2 * N3)
        r[0::2] = z.real.ravel()
        r[1::2] = z.imag.ravel()
        return r
    measure("c3a_DoubleFFT_3D_256_complexForward", f3.plan, N.COMPLEX_FORWARD, buf, 1, 2 * N3, False,
            flops_c2c(N3, 1), 2 * 16 * N3, "5N log2N", ref_fn=fft3)
    del buf
    # config 3b/3c: DoubleDST_3D / DoubleDHT_3D (128^3) uniform[-1, 1)
    N3 = 128 ** 3
    x = torch.from_numpy(rng.uniform(-1, 1, N3)).cuda()
    s3 = J.DoubleDST_3D(128, 128, 128)
    x0 = x.clone()
    measure("c3b_DoubleDST_3D_128_forward", s3.plan, N.FORWARD, x, 1, N3, True,
            2.5 * N3 * math.log2(N3), 2 * 8 * N3, "2.5N log2N",
            ref_fn=lambda a: sfft.dstn(a.reshape(128, 128, 128), type=2, norm="ortho"))
    h3 = J.DoubleDHT_3D(128, 128, 128)
    x.copy_(x0)

    def dht3(a):
        z = np.fft.fftn(a.reshape(128, 128, 128))
        return z.real - z.imag
    measure("c3c_DoubleDHT_3D_128_forward", h3.plan, N.FORWARD, x, 1, N3, False,
            2.5 * N3 * math.log2(N3), 2 * 8 * N3, "2.5N log2N", ref_fn=dht3)
    del x
    out["c5_mixed_batch_10000"] = mixed_batch(args, rng, flush, stream)
    return out


def batch_descriptors(count, rng):
    """(kind, n) of the mixed batch: sizes log-uniform in [16, 65536] redrawn
    into classes (40% powers of two, 40% 2^a 3^b 5^c 7^d, 20% primes); kinds
    50% FloatFFT_1D.complexForward, 25% FloatFFT_1D.realForward, 25%
    DoubleDCT_1D.forward(scale=true)."""
    lo, hi = 16, 65536
    smooth = sorted({2 ** a * 3 ** b * 5 ** c * 7 ** d for a in range(17) for b in range(11) for c in range(8)
                     for d in range(7) if lo <= 2 ** a * 3 ** b * 5 ** c * 7 ** d <= hi})
    sieve = np.ones(hi + 200, bool)
    sieve[:2] = False
    for i in range(2, int((hi + 200) ** 0.5) + 1):
        if sieve[i]:
            sieve[i * i::i] = False
    primes = np.nonzero(sieve)[0]
    primes = primes[(primes >= lo) & (primes <= hi)]
    smooth = np.array(smooth)
    out = []
    for _ in range(count):
        x = math.exp(rng.uniform(math.log(lo), math.log(hi)))
        c = rng.uniform()
        if c < 0.4:
            n = 2 ** int(round(math.log2(x)))
        elif c < 0.8:
            n = int(smooth[np.argmin(np.abs(smooth - x))])
        else:
            n = int(primes[np.argmin(np.abs(primes - x))])
        k = rng.uniform()
        kind = "cf" if k < 0.5 else ("rf" if k < 0.75 else "dct")
        out.append((kind, n))
    return out


def mixed_batch_items(rng):
    """The 10,000 mixed descriptors as batch items over two device buffers:
    (items, items_spec, plans, (b32, b64), flops, desc)."""
    import torch
    from jtransforms_gb300 import _native as N
    desc = batch_descriptors(10000, rng)
    plans = {}
    f32_off, f64_off, items_spec = 0, 0, []
    for kind, n in desc:
        key = (kind, n)
        if key not in plans:
            if kind == "dct":
                plans[key] = N.Plan(N.DCT, N.FLOAT64, [n])
            else:
                plans[key] = N.Plan(N.FFT, N.FLOAT32, [n])
        ext = 2 * n if kind == "cf" else n
        ext = (ext + 3) & ~3  # keep every array 16-byte aligned
        if kind == "dct":
            items_spec.append((key, f64_off, ext))
            f64_off += ext
        else:
            items_spec.append((key, f32_off, ext))
            f32_off += ext
    g = torch.Generator(device="cuda").manual_seed(SEED)
    b32 = torch.rand(max(f32_off, 1), dtype=torch.float32, device="cuda", generator=g) * 2 - 1
    b64 = torch.rand(max(f64_off, 1), dtype=torch.float64, device="cuda", generator=g) * 2 - 1
    opc = {"cf": N.COMPLEX_FORWARD, "rf": N.REAL_FORWARD, "dct": N.FORWARD}
    items = []
    flops = 0.0
    for (kind, n), off, ext in items_spec:
        buf = b64 if kind == "dct" else b32
        ptr = buf.data_ptr() + off * buf.element_size()
        items.append((plans[(kind, n)], opc[kind], ptr, kind == "dct"))
        flops += (5.0 if kind == "cf" else 2.5) * n * math.log2(n)
    return items, items_spec, plans, (b32, b64), flops, desc


def mixed_batch(args, rng, flush, stream):
    import torch
    from jtransforms_gb300 import _native as N
    items, items_spec, plans, (b32, b64), flops, desc = mixed_batch_items(rng)
    p32, p64 = b32.clone(), b64.clone()
    batch = N.Batch(items)

    def restore(i):
        b32.copy_(p32)
        b64.copy_(p64)

    steps, warm = max(args.steps, 20), max(args.warmup, 2)
    t_graph = timed_calls([lambda: batch.run_graph()], restore, flush, steps, warm, stream)[0]
    t_pers = timed_calls([lambda: batch.run()], restore, flush, steps, warm, stream)[0]
    t_each = timed_calls([lambda: batch.run_per_transform()], restore, flush, 5, 1, stream)[0]
    mg, mp, me = statistics.median(t_graph), statistics.median(t_pers), statistics.median(t_each)
    # time per kind and size class: the same descriptors split into batches
    # of one kind (power of two, 7-smooth, Bluestein for the FFT kinds)
    def size_class(n):
        if n & (n - 1) == 0:
            return "pow2"
        m = n
        for p in (2, 3, 5, 7):
            while m % p == 0:
                m //= p
        return "smooth" if m == 1 else "other"
    groups = {}
    for it, ((kind, n), _, _) in zip(items, items_spec):
        groups.setdefault(f"{kind}_{size_class(n)}", []).append((it, (5.0 if kind == "cf" else 2.5) * n * math.log2(n)))
    per_kind = {}
    for name, lst in sorted(groups.items()):
        sub = N.Batch([x[0] for x in lst])
        tk = timed_calls([lambda: sub.run()], restore, flush, steps, warm, stream)[0]
        mk = statistics.median(tk)
        per_kind[name] = {"transforms": len(lst), "ms": mk, "GFLOP/s": sum(x[1] for x in lst) / (mk * 1e-3) / 1e9}
        del sub
    return {"value": len(desc) / (mg * 1e-3), "unit": "transforms/s", "ms": mg,
            "persistent_launch_ms": mp, "per_transform_launches_ms": me,
            "speedup_vs_per_transform": me / mg, "GFLOP/s": flops / (mg * 1e-3) / 1e9,
            "distinct_plans": len(plans), "transforms": len(desc),
            "per_kind_alone": per_kind,
            "flops": "5N log2N complex, 2.5N log2N real and DCT"}


def run_ours(args, world, rank, local):
    import torch
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    torch.cuda.set_device(local)
    if args.no_tma:
        N.set_option(N.OPT_TMA_PIPELINE, 0)
    if args.direct_max:
        N.set_option(N.OPT_DIRECT_MAX_F32, args.direct_max)
    if args.chunk_mb:
        N.set_option(N.OPT_TWOPASS_CHUNK_MB, args.chunk_mb)
    if args.host_piece_mb:
        N.set_option(N.OPT_HOST_PIECE_MB, args.host_piece_mb)
    dist_init(world, "nccl")
    peak, peak_src = measured_peaks()
    stream = torch.cuda.current_stream()
    flushbuf = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def flush():
        flushbuf.fill_(1.0)

    plans, pristine, work = [], [], []
    g = torch.Generator(device="cuda").manual_seed(SEED + rank)
    for n in SIZES:
        plans.append(J.FloatFFT_1D(n))
        p = torch.randn(2 * ELEMS, dtype=torch.float32, device="cuda", generator=g)
        pristine.append(p)
        work.append(torch.empty_like(p))
    torch.cuda.synchronize()

    fns = [(lambda i=i: plans[i].plan.execute(N.COMPLEX_FORWARD, work[i], 0, False,
                                              batch=ELEMS // SIZES[i], dist=2 * SIZES[i]))
           for i in range(len(SIZES))]
    clk = ClockSampler(local).__enter__()  # running before the warm-up: samples cover the timed region
    # warm-up (tables, scratch, clocks)
    timed_calls(fns, lambda i: work[i].copy_(pristine[i]), flush, 0, args.warmup, stream)
    dist_barrier(world)
    torch.cuda.synchronize()
    J.launch_count(reset=True)
    t_wall0 = time.perf_counter()
    times = timed_calls(fns, lambda i: work[i].copy_(pristine[i]), flush, args.steps, 0, stream)
    torch.cuda.synchronize()
    launches = J.launch_count(reset=True)
    t_wall1 = time.perf_counter()
    wall = t_wall1 - t_wall0
    time.sleep(0.1)  # the sample after the window
    clk.__exit__(None, None, None)
    per_size_ms = [sum(t) / len(t) for t in times]
    step_ms = sum(per_size_ms)
    step_ms = max_over_ranks(step_ms, world, "cuda")
    flops_step = sum(flops_c2c(n, ELEMS // n) for n in SIZES) * world
    value = flops_step / (step_ms * 1e-3) / 1e9
    bytes_step = 2 * 8 * ELEMS * len(SIZES)
    achieved = bytes_step / (sum(per_size_ms) * 1e-3) / 1e9
    per_size = {f"2^{int(math.log2(n))}": {"ms": ms, "GFLOP/s": flops_c2c(n, ELEMS // n) / (ms * 1e-3) / 1e9,
                                           "GB/s": 2 * 8 * ELEMS / (ms * 1e-3) / 1e9,
                                           "algorithm": ["direct", "two-pass", "bluestein", "trivial", "three-pass"][plans[i].plan.algorithm(0)]}
                for i, (n, ms) in enumerate(zip(SIZES, per_size_ms))}

    # the output of the last timed call of each size, checked against FP64:
    # the first, middle and last transform of the batch and one drawn at random
    def errs(got_f32, xin_f32):
        x = xin_f32.double()
        ref = torch.fft.fft(torch.complex(x[0::2], x[1::2]))
        got = torch.complex(got_f32[0::2].double(), got_f32[1::2].double())
        d = got - ref
        return (float(torch.linalg.norm(d) / torch.linalg.norm(ref)),
                float(d.abs().max() / ref.abs().max()))

    timed_check = {}
    pick = np.random.default_rng(SEED + 7)
    for i, n in enumerate(SIZES):
        b = ELEMS // n
        worst = [0.0, 0.0]
        ts = sorted({0, b // 2, b - 1, int(pick.integers(0, b))})
        for t in ts:
            e = errs(work[i][2 * n * t: 2 * n * (t + 1)], pristine[i][2 * n * t: 2 * n * (t + 1)])
            worst = [max(worst[0], e[0]), max(worst[1], e[1])]
        timed_check[f"2^{int(math.log2(n))}"] = {"transforms_checked": ts,
                                                 "max_rel_l2_vs_fp64": worst[0], "max_rel_max_err_vs_fp64": worst[1],
                                                 "tol_4eps_log2n": 4 * 2.0 ** -23 * math.log2(n)}

    # error against FP64 of one transform per size: input set (a) = the timed
    # data, set (b) = 60 dB dynamic range; relative L2 and max error
    # (max |got - ref| / max |ref|)
    def rel_err(plan, xin, both=False):
        w = xin.clone()
        plan.execute(N.COMPLEX_FORWARD, w, 0, False)
        e = errs(w, xin)
        return e if both else e[0]

    err, err_b, set_b, err_max, err_b_max = {}, {}, [], {}, {}
    for i, n in enumerate(SIZES):
        set_b.append(sixty_db(n, g))
        key = f"2^{int(math.log2(n))}"
        err[key], err_max[key] = rel_err(plans[i].plan, pristine[i][: 2 * n], True)
        err_b[key], err_b_max[key] = rel_err(plans[i].plan, set_b[i], True)

    # split-operand tensor-core mode beside plain FP32 at every size; the
    # mode's tensor-core kernel covers row passes of 16..2048, longer lengths
    # run the plain passes under it (tc_kernel false)
    tc = {}
    for i, n in enumerate(SIZES):
        plans[i].plan.set_mode(N.MODE_TC_SPLIT)
        tt = timed_calls([fns[i]], lambda _, i=i: work[i].copy_(pristine[i]), flush, max(args.steps, 20), 2, stream)[0]
        ms = statistics.median(tt)
        tc[f"2^{int(math.log2(n))}"] = {
            "ms": ms, "GB/s": 2 * 8 * ELEMS / (ms * 1e-3) / 1e9, "GFLOP/s": flops_c2c(n, ELEMS // n) / (ms * 1e-3) / 1e9,
            "plain_ms": per_size_ms[i], "rel_l2_vs_fp64_a": rel_err(plans[i].plan, pristine[i][: 2 * n]),
            "rel_l2_vs_fp64_b": rel_err(plans[i].plan, set_b[i]),
            "plain_rel_l2_vs_fp64_a": err[f"2^{int(math.log2(n))}"],
            "plain_rel_l2_vs_fp64_b": err_b[f"2^{int(math.log2(n))}"],
            "speed_vs_plain": per_size_ms[i] / ms, "tc_kernel": n <= 2048}
        plans[i].plan.set_mode(N.MODE_FP32)
    del set_b

    # end to end through the C ABI with pinned host buffers
    e2e_val, link = None, None
    del work
    if not args.no_e2e:
        e2e_steps = max(1, min(args.steps, 5))
        host = []
        for i, n in enumerate(SIZES):
            h = torch.empty(2 * ELEMS, dtype=torch.float32, pin_memory=True)
            h.copy_(pristine[i])
            host.append(h.numpy())
        torch.cuda.synchronize()
        for i, n in enumerate(SIZES):  # warm the host path
            plans[i].plan.execute(N.COMPLEX_FORWARD, host[i][: 2 * n * 4], 0, False, batch=4, dist=2 * n)
        step_s = []
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            for i, n in enumerate(SIZES):
                plans[i].plan.execute(N.COMPLEX_FORWARD, host[i], 0, False, batch=ELEMS // n, dist=2 * n)
            step_s.append(time.perf_counter() - t0)
        e2e_s = statistics.median(step_s)  # each call returns after its copies out: wall time is the step
        e2e_val = flops_step / e2e_s / 1e9
        link = link_bandwidth(host[0], pristine[0])
        del host

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": step_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded N(0,1) complex64)",
            "config": headline_config(args),
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak,
                         "traffic": TRAFFIC_PER_STEP * (ELEMS / 2 ** 27) if SIZES == HEADLINE_SIZES else None,
                         "traffic_unit": "bytes per step (DRAM read + write of the five calls)",
                         "peak_source": peak_src,
                         "kernel": "stockham_pipe_kernel / stockham_big_kernel (every launch of the five 1 GiB "
                                   "calls: one pass at 2^10 and 2^14, passes A and B at 2^18..2^24)",
                         "algorithmic_bytes_per_call": 2 * 8 * ELEMS,
                         "algorithmic_bytes_per_step": bytes_step},
            "per_size": per_size, "rel_l2_vs_fp64": err, "rel_l2_vs_fp64_set_b": err_b,
            "rel_max_err_vs_fp64": err_max, "rel_max_err_vs_fp64_set_b": err_b_max,
            "timed_output_check": timed_check,
            "tc_split": {"per_size": tc,
                         "scheme": "radix-16 stages as M128 N32 tcgen05 kind::tf32 products, TF32 head + FP32 remainder, "
                                   "3 products hi*hi + lo*hi + hi*lo, FP32 accumulate in tensor memory; twiddles and "
                                   "the last short radix on CUDA cores",
                         "applies_to": "row passes of length 16..2048 (direct sizes); longer lengths run plain passes "
                                       "under the mode (tc_kernel false)"},
            "e2e": {"value": e2e_val, "unit": UNIT, "h2d_bytes_per_step": 8 * ELEMS * len(SIZES),
                    "d2h_bytes_per_step": 8 * ELEMS * len(SIZES),
                    "path": "FloatFFT_1D plan -> jt_execute_batch on pinned host arrays",
                    "link_GBps": link,
                    "link_bound_GFLOP/s": (flops_step / (8 * ELEMS * len(SIZES) / (link["bidirectional"] / 2 * 1e9)) / 1e9
                                           if link else None)},
            "gpu_launches": launches,
            "timed_wall_s": wall}
    clocks = clk.summary(t_wall0, t_wall1)
    line["clocks"] = clocks
    if rank == 0 and world == 1 and not args.no_cpu:
        v, th, desc = cpu_sample(3.0)
        v1, _, _ = cpu_sample(1.5, threads=1)
        line["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": th, "kind": "port", "sample": desc,
                                "serial_loop": {"value": v1, "unit": UNIT, "cores": 1}}
    if rank == 0 and not args.no_other:
        del pristine
        torch.cuda.empty_cache()
        try:
            line["other_workloads"] = other_workloads(args, peak, flush, stream)
        except Exception as e:  # report, do not hide
            line["other_workloads_error"] = repr(e)
    if rank == 0:
        print(json.dumps(line), flush=True)
    dist_finish(world)
    return 0


def profile_case(case: str) -> int:
    """A small workload for ncu captures: three calls of one transform, then
    (c1) the CUDA-core FMA peaks.  Prints what it ran.  Case `peaks` prints
    the measured FMA and distributed-shared-memory peaks only."""
    import torch
    import jtransforms_gb300 as J
    from jtransforms_gb300 import _native as N
    rng = np.random.default_rng(SEED)
    if case == "peaks":  # measured FMA and distributed-shared-memory peaks, no transform
        lib = N.load()
        for p, name in ((N.FLOAT64, "fp64"), (N.FLOAT32, "fp32")):
            v = ctypes.c_double()
            rc = lib.jt_fma_peak(p, ctypes.byref(v))
            print(f"fma peak {name}: rc {rc}, {v.value:.1f} GFLOP/s")
        for cl in (2, 4, 8, 16):
            for remote in (0, 1):
                v, ctas = ctypes.c_double(), ctypes.c_int()
                rc = lib.jt_dsmem_peak(cl, remote, ctypes.byref(v), ctypes.byref(ctas))
                print(f"dsmem cluster {cl:2d} {'remote' if remote else 'local '}: rc {rc}, "
                      f"{v.value:.1f} GB/s over {ctas.value} CTAs")
        return 0
    if case == "c1":
        n, B = 4096, 256
        plan = J.DoubleFFT_1D(n).plan
        x = torch.from_numpy(rng.uniform(-1, 1, 2 * n * B)).cuda()
        run = lambda: plan.execute(N.COMPLEX_FORWARD, x, 0, False, batch=B, dist=2 * n)  # noqa: E731
    elif case == "c2a":
        plan = J.FloatFFT_2D(2048, 2048).plan
        x = torch.from_numpy(blob_image(2048, rng).astype(np.float32).ravel()).cuda()
        run = lambda: plan.execute(N.REAL_FORWARD, x, 0, False)  # noqa: E731
    elif case == "c2b":
        plan = J.DoubleDCT_2D(1024, 1024).plan
        x = torch.from_numpy(blob_image(1024, rng).ravel()).cuda()
        run = lambda: plan.execute(N.FORWARD, x, 0, True)  # noqa: E731
    elif case == "c3b":
        plan = J.DoubleDST_3D(128, 128, 128).plan
        x = torch.from_numpy(rng.uniform(-1, 1, 128 ** 3)).cuda()
        run = lambda: plan.execute(N.FORWARD, x, 0, True)  # noqa: E731
    elif case == "tile1000":  # DoubleFFT_1D(1000) on 256 MiB: the mixed-radix tile kernel, one pass
        n = 1000
        B = (256 << 20) // (16 * n)
        plan = J.DoubleFFT_1D(n).plan
        x = torch.from_numpy(rng.uniform(-1, 1, 2 * n * B)).cuda()
        run = lambda: plan.execute(N.COMPLEX_FORWARD, x, 0, False, batch=B, dist=2 * n)  # noqa: E731
    elif case == "batch":  # the 10,000 mixed transforms, one persistent launch per call
        items_batch = mixed_batch_items(rng)
        bt = N.Batch(items_batch[0])
        run = lambda: bt.run()  # noqa: E731
    else:  # tc1024: the split tensor-core mode, 2^10 x 2^15 (256 MiB)
        n, B = 1024, 1 << 15
        plan = J.FloatFFT_1D(n).plan
        plan.set_mode(N.MODE_TC_SPLIT)
        x = torch.randn(2 * n * B, dtype=torch.float32, device="cuda")
        run = lambda: plan.execute(N.COMPLEX_FORWARD, x, 0, False, batch=B, dist=2 * n)  # noqa: E731
    for _ in range(3):
        run()
    torch.cuda.synchronize()
    if case == "c1":
        for p, name in ((N.FLOAT64, "fp64"), (N.FLOAT32, "fp32")):
            v = ctypes.c_double()
            rc = N.load().jt_fma_peak(p, ctypes.byref(v))
            print(f"fma peak {name}: rc {rc}, {v.value:.1f} GFLOP/s")
    print(f"case {case}: 3 calls done")
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--no-other", action="store_true", help="skip the other workloads")
    ap.add_argument("--small", action="store_true",
                    help="profiling case: 256 MiB per size instead of 1 GiB, no e2e/CPU/other workloads")
    ap.add_argument("--sizes", type=str, default="", help="comma-separated subset of the headline sizes")
    ap.add_argument("--no-tma", action="store_true", help="use the plain (non-TMA) power-of-two kernel")
    ap.add_argument("--direct-max", type=int, default=0, help="longest float length done in one pass")
    ap.add_argument("--chunk-mb", type=int, default=0, help="MiB of transforms per two-pass chunk (library default 1024)")
    ap.add_argument("--host-piece-mb", type=int, default=0, help="MiB per piece of the end-to-end host batch (library default 64)")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end host-buffer leg")
    ap.add_argument("--case", default="", choices=["", "c1", "c2a", "c2b", "c3b", "tc1024", "tile1000", "batch", "peaks"],
                    help="profiling case: run one small workload a few times and exit (no JSON line)")
    args = ap.parse_args()
    global ELEMS, SIZES
    if args.small:
        ELEMS = 2 ** 25
        args.no_cpu = args.no_other = True
        args.no_e2e = True
    if args.sizes:
        SIZES = [int(s) for s in args.sizes.split(",")]
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world, rank, local = dist_setup(args)
    if args.case:
        if args.no_tma:
            from jtransforms_gb300 import _native as N
            N.set_option(N.OPT_TMA_PIPELINE, 0)
        return profile_case(args.case)
    if args.impl == "reference":
        return run_reference(args, world, rank)
    return run_ours(args, world, rank, local)


if __name__ == "__main__":
    sys.exit(main())

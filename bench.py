#!/usr/bin/env python3
"""Benchmark of the GB300 Winograd 3x3 conv2d operator.

Default workload: N=32, C=256, H=W=56, K=256, 3x3, pad 1, stride 1, fp16
NCHW input ~U[-1,1] and fp16 filter ~N(0, std 1/sqrt(9C)) from a fixed seed,
run through the operator's C ABI with the per-shape autotuner's algorithm
(--algo ref gives the reference's selection rule, F(2x3) fused here).

One step = one conv2d call over one batch.  `value` is effective TFLOP/s
(direct-convolution FLOPs 2*N*K*OH*OW*C*9 / time) with inputs resident in
HBM; `e2e` is the same metric through the host-buffer C entry point
(conv2d_fp16_host: pinned input copied in, output copied out, every step).
Buffer sets rotate so the bytes touched between two uses of one set exceed
the 129 MB L2.  The line also carries the metric's comparison: the
24-problem batch grouped vs per-call (`batched`), a bounded request trace
through the continuous-batching server vs the plain per-call path
(`served`), both summarised in `served_vs_percall`, and the relative error
of the timed output against FP64 (`rel_err`).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload cfg2|cfg1|cfg3|...] [--algo ref|fused|2x3|4x3|row|auto]
"""
from __future__ import annotations

import argparse
import importlib.util
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
METRIC = "3x3 conv eff. TFLOP/s, p50/p99 latency: served vs per-call at fixed rel err"
L2_BYTES = 129 * 1024 * 1024

# (n, c, h, w, k, input distribution, filter distribution, description)
WORKLOADS = {
    "cfg2": (32, 256, 56, 56, 256, "uniform", "normal",
             "single-shape workload N=32 C=256 H=W=56 K=256, 3x3 pad 1 stride 1, fp16 NCHW (configured as "
             "F(2x3) fused and non-fused: both reported under f2x3; the headline runs the autotuner's choice)"),
    "cfg1": (1, 64, 56, 56, 64, "uniform", "uniform",
             "small workload: N=1 C=64 H=W=56 K=64, 3x3 pad 1 stride 1, fp16 NCHW"),
    "cfg3": (32, 512, 28, 28, 512, "normal", "normal",
             "precision-study shape: N=32 C=512 H=W=28 K=512, 3x3 pad 1 stride 1, fp16 NCHW"),
    "final1": (16, 128, 64, 64, 27, "uniform", "uniform", "contest shape 16x128x64x64 -> 27"),
    "final2": (16, 256, 32, 32, 256, "uniform", "uniform", "contest shape 16x256x32x32 -> 256"),
    "final3": (16, 64, 128, 128, 64, "uniform", "uniform", "contest shape 16x64x128x128 -> 64"),
    "final4": (2, 1920, 32, 32, 640, "uniform", "uniform", "contest shape 2x1920x32x32 -> 640"),
    "final5": (2, 640, 64, 64, 640, "uniform", "uniform", "contest shape 2x640x64x64 -> 640"),
    "final6": (2, 320, 64, 64, 4, "uniform", "uniform", "contest shape 2x320x64x64 -> 4"),
    "pre1": (64, 256, 14, 14, 256, "uniform", "uniform", "contest shape 64x256x14x14 -> 256"),
    "pre2": (256, 192, 14, 14, 192, "uniform", "uniform", "contest shape 256x192x14x14 -> 192"),
    "pre3": (16, 256, 26, 26, 512, "uniform", "uniform", "contest shape 16x256x26x26 -> 512"),
    "pre4": (32, 256, 14, 14, 256, "uniform", "uniform", "contest shape 32x256x14x14 -> 256"),
    "pre5": (2, 1280, 16, 16, 1280, "uniform", "uniform", "contest shape 2x1280x16x16 -> 1280"),
    "pre6": (2, 960, 64, 64, 32, "uniform", "uniform", "contest shape 2x960x64x64 -> 32"),
}
# reference latencies read from its published chart (Hygon DCU gfx928), microseconds
PUBLISHED_US = {"final1": 207, "final2": 367, "final3": 724, "final4": 654, "final5": 593, "final6": 133}
ALGO_ARG = {"ref": -1, "4x3": 0, "2x3": 1, "fused": 2, "auto": 3, "row": 4}
SERVE_WORKLOADS = {
    "cfg5": "serving: 16 resident 3x3 pad-1 layers (C,K in {64..512}, H=W in {7..112}), N ~ U{1..64}, "
            "Poisson arrivals swept over multiples of the plain per-request capacity, 40 GiB workspace budget",
}
BATCH_WORKLOADS = {
    "cfg4": "24 uneven 3x3 pad-1 problems in one grouped graph launch: C,K in {64,128,256,512}, "
            "H=W in {7,14,28,56,112}, N in {1,...,128}, U[-1,1], seed 20261203",
}


def batch_shapes(seed=20261203, count=24):
    """The seeded draw of the batched workload: (n, c, h, k) per problem."""
    import numpy as np
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        c = int(rng.choice([64, 128, 256, 512]))
        k = int(rng.choice([64, 128, 256, 512]))
        h = int(rng.choice([7, 14, 28, 56, 112]))
        n = int(rng.choice([1, 2, 4, 8, 16, 32, 64, 128]))
        out.append((n, c, h, k))
    return out


FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}


def load_pkg():
    if "wgconv" in sys.modules:
        return sys.modules["wgconv"]
    spec = importlib.util.spec_from_file_location("wgconv", os.path.join(ROOT, "dcu-winograd-conv2d_gb300",
                                                                         "__init__.py"))
    mod = importlib.util.module_from_spec(spec)
    sys.modules["wgconv"] = mod
    spec.loader.exec_module(mod)
    return mod


def load_oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # noqa: E402
    return oracle


def direct_flops(n, c, h, w, k, p=1, q=1):
    return 2.0 * n * k * (h + 2 * p - 2) * (w + 2 * q - 2) * c * 9


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    except (OSError, ValueError):
        return dict(FALLBACK_PEAKS), "fallback"


def env_dist():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ---- clocks sampler ------------------------------------------------------------

class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.proc = None
        self.path = None
        self.dev = device_index

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(prefix="clocks_", suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.fh.close()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for nm, val in zip(names, r[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(rows)}


def with_window(clocks):
    if clocks is not None:
        clocks["window"] = "0.6 s of untimed steps of the same work, then the timed steps"
    return clocks


def load_phase(step, device, seconds=0.6):
    """Untimed steps of the benchmark's own work for `seconds`, so that the
    clock samples (200 ms apart) see the GPU under the load the timed steps
    then put on it; the timed steps follow at once."""
    import torch

    t0 = time.perf_counter()
    i = 0
    while time.perf_counter() - t0 < seconds:
        for _ in range(16):
            step(i)
            i += 1
        torch.cuda.synchronize(device)


# ---- CPU baseline (the reference verifier or its port) -------------------------

def cpu_sample(O, x16, w16, n_img, threads):
    """Direct conv of `n_img` images on `threads` host threads.  Uses the
    reference's own conv2dcpu (oracle/_ref) when that build loads here, else
    the oracle's C port of it.  Returns (seconds, flops, kind)."""
    import concurrent.futures as cf
    import numpy as np
    xs = np.ascontiguousarray(x16[:n_img])
    n, c, h, w = xs.shape
    k = w16.shape[0]
    flops = direct_flops(n, c, h, w, k)
    if O.ref_lib() is not None:
        # split output channels across threads; each call is the unmodified function
        ksplit = max(1, min(threads, k))
        bounds = [(k * i // ksplit, k * (i + 1) // ksplit) for i in range(ksplit)]
        parts = [np.ascontiguousarray(w16[a:b]) for a, b in bounds]
        t0 = time.perf_counter()
        with cf.ThreadPoolExecutor(max_workers=ksplit) as ex:
            list(ex.map(lambda wt: O.ref_conv2dcpu(xs, wt), parts))
        return time.perf_counter() - t0, flops, "reference", ksplit
    t0 = time.perf_counter()
    O.conv2d_direct(xs, w16, nthreads=threads, want64=False)
    return time.perf_counter() - t0, flops, "port", threads


def replica_throughput(local_ms, flops_per_step, steps, world, dist, device):
    """Replicas only: every rank runs the same workload on its own GPU with no
    data-path exchange.  The job's time is the slowest rank's (MAX over ranks)
    and `value` counts the work of all ranks: world * flops * steps / time."""
    import torch
    total_ms = float(local_ms)
    if dist is not None and world > 1:
        tt = torch.tensor([total_ms], device=device)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    return total_ms, world * flops_per_step * steps / (total_ms * 1e-3) / 1e12


def reference_arm(args):
    """--impl reference: the reference's CPU implementation of the path on the
    host cores, same workload/metric; each step is a bounded sample."""
    import numpy as np
    rank, world, _ = env_dist()
    if rank != 0:
        return 0
    O = load_oracle()
    if not os.path.exists(O.LIB_PATH):
        O.build()
    n, c, h, w, k, xdist, wdist, desc = WORKLOADS[args.workload]
    rng_x, rng_w = sample_host_inputs(O, args.workload, n_img=1)
    threads = os.cpu_count() or 1
    times = []
    kind = None
    used = threads
    for i in range(args.warmup + args.steps):
        dt, fl, kind, used = cpu_sample(O, rng_x, rng_w, 1, threads)
        if i >= args.warmup:
            times.append(dt)
    mean = sum(times) / len(times)
    val = fl / mean / 1e12
    sample = f"1 of {n} images ({fl / 1e9:.2f} GFLOP) per step, all {k} output channels"
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f16", "data": "synthetic (seeded)",
        "config": {"workload": desc, "n": n, "c": c, "h": h, "w": w, "k": k, "pad": 1, "stride": 1},
        "cpu_baseline": {"value": val, "unit": "TFLOP/s", "cores": used, "kind": kind, "sample": sample},
        "e2e": {"value": val, "unit": "TFLOP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def sample_host_inputs(O, workload, n_img):
    """Seeded host copy of the first `n_img` images of the workload (and the filter)."""
    n, c, h, w, k, xdist, wdist, _ = WORKLOADS[workload]
    import numpy as np
    rng = np.random.default_rng(20261203)
    if xdist == "normal":
        x = rng.standard_normal((n_img, c, h, w)).astype(np.float16)
    else:
        x = rng.uniform(-1, 1, size=(n_img, c, h, w)).astype(np.float16)
    if wdist == "normal":
        wt = (rng.standard_normal((k, c, 3, 3)) / math.sqrt(9 * c)).astype(np.float16)
    else:
        wt = rng.uniform(-1, 1, size=(k, c, 3, 3)).astype(np.float16)
    return x, wt


# ---- our arm ---------------------------------------------------------------------

def make_inputs(torch, workload, device, seed):
    n, c, h, w, k, xdist, wdist, _ = WORKLOADS[workload]
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    if xdist == "normal":
        x = torch.randn((n, c, h, w), generator=g, device=device, dtype=torch.float32).half()
    else:
        x = (torch.rand((n, c, h, w), generator=g, device=device, dtype=torch.float32) * 2 - 1).half()
    if wdist == "normal":
        wt = (torch.randn((k, c, 3, 3), generator=g, device=device) / math.sqrt(9 * c)).half()
    else:
        wt = (torch.rand((k, c, 3, 3), generator=g, device=device) * 2 - 1).half()
    return x, wt


def algorithmic_work(name, geo, m_bytes_per_value=None):
    """Per-launch work of one kernel (P tiles, E = (m+2)^2 Winograd elements,
    fp16 tensors and operands).

    Algorithmic bytes are the per-unit figures of the hot path's measurement
    table: what a kernel must move whatever its design.  The GEMM's are V and
    U; its fp32 M is not counted, since an epilogue that applied A^T m A would
    keep M on chip, and the output transform's are the output y alone.  M is
    reported separately as `design_bytes` (the bytes this three-kernel design
    moves), so the difference shows what the unfused M costs.
      input_transform   x (2*N*C*H*W) + V (2*E*P*C)
      gemm_tcgen05      V + U (2*E*C*K);            FLOPs 2*E*P*C*K
      output_transform  y (2*N*K*OH*OW)
      fused2x3          x + U + y;                   FLOPs 2*16*P*C*K
      row4x3            x + U1 (2*18*C*K) + y;       FLOPs 2*18*RT*C*K over
                        RT = N*OH*ceil(OW/4) row tiles
    M is counted at `m_bytes_per_value` bytes per value (3 for the 24-bit
    F(4x3) default, stored in blocks of 64 tiles; 4 for fp32, 2 for fp16).
    Returns (algorithmic bytes, design bytes, FLOPs, formula)."""
    n, c, h, w, k, m = geo
    oh, ow = h, w  # pad 1
    tiles = n * math.ceil(oh / m) * math.ceil(ow / m)
    E = (m + 2) ** 2
    mb = m_bytes_per_value or (3.0 if m == 4 else 2.0)
    x_b, y_b = 2.0 * n * c * h * w, 2.0 * n * k * oh * ow
    m_tiles = math.ceil(tiles / 64) * 64 if mb == 3.0 else tiles
    v_b, u_b, m_b = 2.0 * E * tiles * c, 2.0 * E * c * k, mb * E * m_tiles * k
    if name == "gemm_tcgen05":
        return v_b + u_b, v_b + u_b + m_b, 2.0 * E * tiles * c * k, f"V + U (design adds M {m_b / 1e6:.1f} MB)"
    if name == "fused2x3":
        return x_b + u_b + y_b, x_b + u_b + y_b, 2.0 * E * tiles * c * k, "x + U + y"
    if name == "row4x3":
        rt = n * oh * math.ceil(ow / 4)
        u1 = 2.0 * 18 * c * k
        return x_b + u1 + y_b, x_b + u1 + y_b, 2.0 * 18 * rt * c * k, "x + U1 + y"
    if name == "input_transform":
        return x_b + v_b, x_b + v_b, 0.0, "x + V"
    if name == "tile_scale":
        return x_b, x_b, 0.0, "x"
    return y_b, m_b + y_b, 0.0, f"y (design adds M {m_b / 1e6:.1f} MB)"


def roofline_for(name, wg, geo, ms, pk, pk_kind, m_bytes_per_value=None):
    """Roofline of one kernel from its algorithmic work per launch and its
    CUDA-event duration `ms`.  A kernel with FLOPs is bound by the roof its
    arithmetic intensity puts it under (machine balance = peak FLOP/s / peak
    bytes/s); `frac` is the bound's time over the measured time, i.e. the
    larger of the two fractions."""
    byts, design, flops, formula = algorithmic_work(name, geo, m_bytes_per_value)
    peak_bw, peak_fl = pk["hbm_gbs"], pk["bf16_tflops"]
    out = {"kernel": name}
    if flops and flops / byts > peak_fl * 1e12 / (peak_bw * 1e9):
        ach = flops / (ms * 1e-3) / 1e12
        out.update({"bound": "tensor", "achieved": ach, "peak": peak_fl, "unit": "TFLOP/s", "frac": ach / peak_fl,
                    "peak_source": f"{pk_kind} bf16 dense (burst)"})
    else:
        ach = byts / (ms * 1e-3) / 1e9
        out.update({"bound": "hbm", "achieved": ach, "peak": peak_bw, "unit": "GB/s", "frac": ach / peak_bw,
                    "peak_source": f"{pk_kind} HBM copy"})
    E = (geo[5] + 2) ** 2
    out["algorithmic_per_launch"] = f"{byts / 1e6:.1f} MB ({formula})" + (
        (f", {flops / 1e9:.2f} GFLOP (2*18*RT*C*K)" if name == "row4x3" else f", {flops / 1e9:.2f} GFLOP (2*{E}*P*C*K)")
        if flops else "")
    out["algorithmic_bytes"] = byts
    out["design_bytes"] = design
    out["design_bytes_frac"] = design / (ms * 1e-3) / 1e9 / peak_bw
    if flops:
        out["tensor_frac"] = flops / (ms * 1e-3) / 1e12 / peak_fl
        out["hbm_frac"] = byts / (ms * 1e-3) / 1e9 / peak_bw
    out["launch_us"] = ms * 1e3
    return out


def step_roofline(geo, algo, wg, ms_step, pk, pk_kind):
    """Whole-step roofline of one call: the bytes no design can avoid (x, the
    transformed filter U, y) and the algorithm's tensor work (its Winograd
    GEMM FLOPs), against the measured time per step."""
    n, c, h, w, k, m = geo
    tiles = n * math.ceil(h / m) * math.ceil(w / m)
    E = (m + 2) ** 2
    x_b, y_b = 2.0 * n * c * h * w, 2.0 * n * k * h * w
    if algo == wg.ALGO_4X3_ROW:
        u_b, flops = 2.0 * 18 * c * k, 2.0 * 18 * n * h * math.ceil(w / 4) * c * k
    else:
        u_b, flops = 2.0 * E * c * k, 2.0 * E * tiles * c * k
    t_bytes = (x_b + u_b + y_b) / (pk["hbm_gbs"] * 1e9)
    t_flops = flops / (pk["bf16_tflops"] * 1e12)
    return {"bytes": x_b + u_b + y_b, "formula": "x + U + y", "flops": flops,
            "bound": "hbm" if t_bytes >= t_flops else "tensor",
            "floor_us": max(t_bytes, t_flops) * 1e6, "ms_per_step": ms_step,
            "frac": max(t_bytes, t_flops) / (ms_step * 1e-3), "peak_source": pk_kind}


def rel_err_slice(x, wt, y, nhwc, tol, channels=8):
    """Max / mean relative error of the operator's output against an FP64
    direct convolution (pad 1) of image 0 at `channels` output channels
    spread over K: |y - ref| / max(|ref|, rms(ref)), the parity tests'
    measure, with the tolerance it is held to."""
    import numpy as np
    x0 = x[0].float().cpu().numpy().astype(np.float64)
    if nhwc:
        x0 = x0.transpose(2, 0, 1)
    C, H, W = x0.shape
    K = wt.shape[0]
    ks = sorted({int(round(i * (K - 1) / max(1, channels - 1))) for i in range(channels)})
    w64 = wt.float().cpu().numpy().astype(np.float64)[ks]
    xp = np.zeros((C, H + 2, W + 2))
    xp[:, 1:H + 1, 1:W + 1] = x0
    ref = np.zeros((len(ks), H, W))
    for r in range(3):
        for s_ in range(3):
            ref += np.tensordot(w64[:, :, r, s_], xp[:, r:r + H, s_:s_ + W], axes=([1], [0]))
    y0 = y[0].float().cpu().numpy().astype(np.float64)
    y0 = y0[:, :, ks].transpose(2, 0, 1) if nhwc else y0[ks]
    rms = math.sqrt(float(np.mean(ref * ref)))
    rel = np.abs(y0 - ref) / np.maximum(np.abs(ref), rms)
    mx = float(rel.max())
    return {"max": mx, "mean": float(rel.mean()), "tol": tol, "within_tol": bool(mx <= tol),
            "against": f"FP64 direct convolution of image 0, output channels {ks}",
            "measure": "|y - ref| / max(|ref|, rms(ref))"}


def f2x3_paths(wg, torch, xs, ys, wt, geo, sptr, device, reps, pk, pk_kind):
    """The F(2x3) paths (non-fused and fused) on the same buffer sets as the
    headline run: effective TFLOP/s per call (back-to-back calls) and, per
    kernel, its roofline: HBM GB/s for the transforms, tensor-pipe share for
    the 16 batched C x K GEMMs.  A failure is reported, not raised."""
    n, c, h, w, k = geo
    flops = direct_flops(n, c, h, w, k)
    out = {}
    for label, algo in (("non_fused", wg.ALGO_2X3), ("fused", wg.ALGO_2X3_FUSED)):
        ops = []
        try:
            for x, y in zip(xs, ys):
                prob = wg.make_problem(x.data_ptr(), wt.data_ptr(), y.data_ptr(), n, c, h, w, k)
                ops.append(wg.Conv2d(prob, wg.default_options(algo=algo)))
            for i in range(3):
                ops[i % len(ops)](sptr)
            torch.cuda.synchronize(device)
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            stream = torch.cuda.current_stream(device)
            a.record(stream)
            for i in range(reps):
                ops[i % len(ops)](sptr)
            b.record(stream)
            torch.cuda.synchronize(device)
            ms = a.elapsed_time(b) / reps
            kt = {}
            for i in range(reps):
                for nm, t in zip(ops[0].kernel_names(), ops[i % len(ops)].timed(sptr)):
                    kt.setdefault(nm, []).append(t)
            kernels = {}
            for nm, v in kt.items():
                r = roofline_for(nm, wg, (n, c, h, w, k, 2), sum(v) / len(v), pk, pk_kind)
                kernels[nm] = {key: r[key] for key in ("launch_us", "bound", "achieved", "unit", "frac",
                                                      "algorithmic_per_launch", "tensor_frac", "hbm_frac",
                                                      "design_bytes_frac") if key in r}
            ok = all(op.check_device()[0] == wg.OK for op in ops)
            out[label] = {"value": flops / (ms * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_call": ms,
                          "calls": reps, "kernels": kernels, "device_ok": ok}
        except Exception as e:  # reported beside the headline, which stands on its own
            out[label] = {"error": f"{type(e).__name__}: {e}"[:300]}
        finally:
            for op in ops:
                op.destroy()
    return out


def committed_traffic(kernel, workload):
    """DRAM bytes per launch recorded from an ncu capture in profiles/ (a line
    `traffic <kernel> <workload> <bytes>` in profiles/traffic.txt), else None."""
    path = os.path.join(ROOT, "profiles", "traffic.txt")
    try:
        with open(path) as f:
            for line in f:
                parts = line.split()
                if len(parts) >= 4 and parts[0] == "traffic" and parts[1] == kernel and parts[2] == workload:
                    return float(parts[3])
    except OSError:
        pass
    return None


def our_arm(args):
    import numpy as np
    import torch

    rank, world, local = env_dist()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    wg = load_pkg()
    wg.lib()  # the CUDA library must load; there is no fallback
    n, c, h, w, k, xdist, wdist, desc = WORKLOADS[args.workload]
    flops = direct_flops(n, c, h, w, k)

    opts = wg.default_options(algo=ALGO_ARG[args.algo])
    if args.gemm_bn:
        opts.gemm_bn = args.gemm_bn
    if args.l2_chunk is not None:
        opts.l2_chunk_bytes = args.l2_chunk
    if args.nhwc:
        opts.layout_nhwc = 1
    if args.m_fp32:
        opts.m_fp32 = 1
    in_bytes = 2 * n * c * h * w
    out_bytes = 2 * n * k * h * w
    nsets = max(2, math.ceil(3 * L2_BYTES / (in_bytes + out_bytes)))
    nsets = min(nsets, 16)
    xs, ys, ops = [], [], []
    x0, wt = make_inputs(torch, args.workload, device, seed=1234 + rank)
    for i in range(nsets):
        x = x0 if i == 0 else x0.roll(i, dims=0).contiguous()
        if args.nhwc:  # the same values, channels last
            x = x.permute(0, 2, 3, 1).contiguous()
        y = torch.empty((n, h, w, k) if args.nhwc else (n, k, h, w), dtype=torch.float16, device=device)
        prob = wg.make_problem(x.data_ptr(), wt.data_ptr(), y.data_ptr(), n, c, h, w, k)
        xs.append(x)
        ys.append(y)
        ops.append(wg.Conv2d(prob, opts))
    stream = torch.cuda.current_stream(device)
    sptr = stream.cuda_stream
    algo = ops[0].algo

    for i in range(args.warmup):
        ops[i % nsets](sptr)
    torch.cuda.synchronize(device)
    st, site = ops[0].check_device()
    if st != wg.OK:
        raise RuntimeError(f"device wait gave up at site {site}")

    sampler = ClockSampler(local)
    sampler.start()
    load_phase(lambda i: ops[i % nsets](sptr), device)
    if dist:
        dist.barrier()
    torch.cuda.synchronize(device)
    # the timed steps are queued back to back with events only at the two
    # ends: an event between two calls would keep the next call's first kernel
    # from being scheduled behind the previous call's last one
    t_start = torch.cuda.Event(enable_timing=True)
    t_end = torch.cuda.Event(enable_timing=True)
    t_start.record(stream)
    for i in range(args.steps):
        ops[i % nsets](sptr)
    t_end.record(stream)
    torch.cuda.synchronize(device)
    if dist:
        dist.barrier()
    # per-call latency (p50 / p99): the same calls again, each between events
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    for i in range(args.steps):
        evs[i][0].record(stream)
        ops[i % nsets](sptr)
        evs[i][1].record(stream)
    torch.cuda.synchronize(device)
    clocks = with_window(sampler.stop())
    per_step = [a.elapsed_time(b) for a, b in evs]
    total_ms, value = replica_throughput(t_start.elapsed_time(t_end), flops, args.steps, world, dist, device)
    ms_per_step = total_ms / args.steps

    # per-kernel durations (CUDA events between the launches of one call)
    names = ops[0].kernel_names()
    kt = {}
    reps = min(args.steps, 20)
    for i in range(reps):
        d = ops[i % nsets].timed(sptr)
        for nm, ms in zip(names, d):
            kt.setdefault(nm, []).append(ms)
    tot = {nm: sum(v) for nm, v in kt.items()}
    dominant = max(tot, key=tot.get)
    launches_of_dom = len(kt[dominant])
    dom_ms = tot[dominant] / launches_of_dom
    m = 4 if algo in (wg.ALGO_4X3, wg.ALGO_4X3_ROW) else 2
    pk, pk_kind = peaks()
    mbv = 2.0 if m == 2 else (4.0 if args.m_fp32 else 3.0)
    roof = roofline_for(dominant, wg, (n, c, h, w, k, m), dom_ms, pk, pk_kind, mbv)
    traffic = committed_traffic(dominant, args.workload)
    roof["traffic"] = traffic
    roof["traffic_over_algorithmic"] = traffic / roof["algorithmic_bytes"] if traffic else None
    roof["share_of_step"] = tot[dominant] / max(1e-9, sum(tot.values()))
    roof["step"] = step_roofline((n, c, h, w, k, m), algo, wg, ms_per_step, pk, pk_kind)
    kernel_ms = {nm: sum(v) / len(v) * (len(v) / reps) for nm, v in kt.items()}
    kernel_roofline = {nm: {key: r[key] for key in ("bound", "frac", "hbm_frac", "tensor_frac", "design_bytes_frac",
                                                  "algorithmic_per_launch") if key in r}
                       for nm, r in ((nm, roofline_for(nm, wg, (n, c, h, w, k, m), sum(kt[nm]) / len(kt[nm]), pk,
                                                       pk_kind, mbv)) for nm in kt)}

    # accuracy of what was timed: the last timed step's output against FP64
    last = (args.steps - 1) % nsets
    rel_err = rel_err_slice(xs[last], wt, ys[last], args.nhwc, 2e-2 if m == 4 else 1e-2)

    # the workload names F(2x3), fused and non-fused: both measured beside the
    # autotuned headline, on the same buffers
    f2x3 = None
    if args.workload == "cfg2" and not args.nhwc and world == 1:
        f2x3 = f2x3_paths(wg, torch, xs, ys, wt, (n, c, h, w, k), sptr, device, reps, pk, pk_kind)

    # end to end through the host-buffer entry points: every step copies its
    # input in from pinned host memory and its output back out
    e2e = None
    if not args.no_e2e:
        hins = [torch.empty(tuple(xs[0].shape), dtype=torch.float16).pin_memory() for _ in range(2)]
        for hb, src in zip(hins, xs[:2]):
            hb.copy_(src.cpu())
        houts = [torch.empty(tuple(ys[0].shape), dtype=torch.float16).pin_memory() for _ in range(2)]
        e_steps = max(3, min(args.steps, 20))
        ins = [hins[i % 2].data_ptr() for i in range(e_steps)]
        outs = [houts[i % 2].data_ptr() for i in range(e_steps)]
        for i in range(2):
            ops[0].host(ins[i], outs[i], sptr)
        ops[0].host_steps(ins[:3], outs[:3], sptr)
        torch.cuda.synchronize(device)

        def wall(fn):
            if dist:
                dist.barrier()
            t0 = time.perf_counter()
            fn()
            el = time.perf_counter() - t0
            if dist:
                tt = torch.tensor([el], device=device)
                dist.all_reduce(tt, op=dist.ReduceOp.MAX)
                el = float(tt.item())
            return el

        # one pipelined call over the e_steps batches (conv2d_fp16_host_steps)
        el = wall(lambda: ops[0].host_steps(ins, outs, sptr))
        # one blocking call per batch (conv2d_fp16_host)
        el1 = wall(lambda: [ops[0].host(ins[i], outs[i], sptr) for i in range(e_steps)])
        e2e = {"value": world * flops * e_steps / el / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": in_bytes,
               "d2h_bytes_per_step": out_bytes, "ms_per_step": el / e_steps * 1e3, "steps": e_steps,
               "path": "conv2d_fp16_host_steps: consecutive pinned host batches in one call, each copied in and "
                       "out in full, copies of consecutive batches overlapping",
               "per_call": {"value": world * flops * e_steps / el1 / 1e12, "ms_per_step": el1 / e_steps * 1e3,
                            "path": "conv2d_fp16_host: one blocking call per batch (stream sync per call)"}}

    # CPU baseline on the host cores (rank 0 of a 1-GPU run only)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        O = load_oracle()
        if not os.path.exists(O.LIB_PATH):
            O.build()
        hx, hw = sample_host_inputs(O, args.workload, n_img=1)
        threads = os.cpu_count() or 1
        dt, fl, kind, used = cpu_sample(O, hx, hw, 1, threads)
        cpu = {"value": fl / dt / 1e12, "unit": "TFLOP/s", "cores": used, "kind": kind,
               "sample": f"1 of {n} images ({fl / 1e9:.2f} GFLOP), all {k} output channels, {dt:.2f} s"}

    cudnn = None
    if not args.no_cudnn:
        if args.nhwc:  # cuDNN's channels-last kernels on the same values
            cx, cw = x0.contiguous(memory_format=torch.channels_last), wt.contiguous(memory_format=torch.channels_last)
        else:
            cx, cw = xs[0], wt
        cms = time_cudnn(torch, cx, cw, args.steps, args.warmup)
        cudnn = {"value": flops / (cms * 1e-3) / 1e12, "unit": "TFLOP/s", "ms_per_step": cms,
                 "path": f"torch.nn.functional.conv2d fp16 {'NHWC' if args.nhwc else 'NCHW'}, cudnn.benchmark"}
    # the metric's comparison: batched and served runs against plain per-call
    # launches of the same kernels, at the error the single-shape run holds
    batched = served = None
    launches_per_call = ops[0].launches_per_call
    if args.workload == "cfg2" and not args.nhwc and world == 1 and not args.no_serving:
        for op in ops:
            op.destroy()
        ops = []
        try:
            batched, _, _ = batched_run(wg, torch, device, max(5, min(args.steps, 20)), args.warmup)
        except Exception as e:  # reported beside the headline, which stands on its own
            batched = {"error": f"{type(e).__name__}: {e}"[:300]}
        try:
            served, _ = serving_run(wg, torch, device, args.line_requests, [0.9])
        except Exception as e:
            served = {"error": f"{type(e).__name__}: {e}"[:300]}
    precision = None
    if args.workload == "cfg2" and world == 1 and not args.no_precision:
        for op in ops:
            op.destroy()
        ops = []
        try:
            precision = precision_line(wg, torch, device)
        except Exception as e:
            precision = {"error": f"{type(e).__name__}: {e}"[:300]}
    served_vs_percall = None
    if batched or served:
        served_vs_percall = {
            "batched_24_problems": (batched or {}).get("grouped_over_percall"),
            "served_saturated": ((served or {}).get("saturated") or {}).get("served_over_plain"),
            "served_p50_p99_us_at_0.9_plain_capacity":
                [(served or {}).get("sweep", [{}])[0].get("served", {}).get(k) for k in ("p50_us", "p99_us")]
                if served and "sweep" in served else None,
            "plain_p50_p99_us_at_0.9_plain_capacity":
                [(served or {}).get("sweep", [{}])[0].get("plain", {}).get(k) for k in ("p50_us", "p99_us")]
                if served and "sweep" in served else None,
            "rel_err_max": rel_err["max"], "rel_err_tol": rel_err["tol"],
            "target": ">= 1.5x plain per-call throughput at the stated error bound",
        }
    lat = sorted(per_step)
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f16", "data": "synthetic (seeded torch RNG)",
        "config": {"workload": desc, "n": n, "c": c, "h": h, "w": w, "k": k, "pad": 1, "stride": 1,
                   "algo": wg.ALGO_NAMES[algo], "selection": args.algo, "accumulate": "fp32",
                   "input": f"{xdist}, filter {wdist}",
                   "l2": f"{nsets} rotating input/output sets ({nsets * (in_bytes + out_bytes) / 2**20:.0f} MiB) > L2",
                   "timing": "K calls back to back, CUDA events at the two ends; latency_us from a second pass "
                             "with events around each call",
                   "layout": "NHWC" if args.nhwc else "NCHW",
                   "m_storage": "fp32" if args.m_fp32 else "24-bit (F(4x3)) / fp16 (F(2x3))",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "latency_us": {"p50": lat[len(lat) // 2] * 1e3, "p99": lat[min(len(lat) - 1, int(0.99 * len(lat)))] * 1e3},
        "kernel_ms": kernel_ms,
        "kernel_roofline": kernel_roofline,
        "roofline": roof,
        "rel_err": rel_err,
        "e2e": e2e,
        "cpu_baseline": cpu,
        "cudnn": cudnn,
        "f2x3": f2x3,
        "served_vs_percall": served_vs_percall,
        "batched": batched,
        "served": served,
        "precision": precision,
        "clocks": clocks,
        "gpu_launches": args.steps * launches_per_call,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    for op in ops:
        op.destroy()
    if dist:
        dist.destroy_process_group()
    return 0


def batched_run(wg, torch, device, steps, warmup, algo=3, seed=99, with_e2e=False):
    """The 24-problem batch: every problem in one grouped run (grouped
    launches replayed from a CUDA graph) against the same problems launched
    one conv2d call after another on the same stream (the per-call path).
    Returns a summary dict (and the clock record of the grouped steps)."""
    shapes = batch_shapes()
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    probs, keep = [], []
    flops = 0.0
    in_bytes = out_bytes = 0
    for n, c, h, k in shapes:
        x = (torch.rand((n, c, h, h), generator=g, device=device) * 2 - 1).half()
        w = (torch.rand((k, c, 3, 3), generator=g, device=device) * 2 - 1).half()
        y = torch.empty((n, k, h, h), dtype=torch.float16, device=device)
        probs.append(wg.make_problem(x.data_ptr(), w.data_ptr(), y.data_ptr(), n, c, h, h, k))
        keep.append((x, w, y))
        flops += direct_flops(n, c, h, h, k)
        in_bytes += x.numel() * 2
        out_bytes += y.numel() * 2
    t0 = time.perf_counter()
    batch = wg.Batch(probs, wg.default_options(algo=algo))
    setup_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(device)
    sptr = stream.cuda_stream
    for _ in range(warmup):
        batch.run(sptr)
        batch.run_percall(sptr)
    torch.cuda.synchronize(device)
    st, site = batch.check_device()
    if st != wg.OK:
        raise RuntimeError(f"device wait gave up at site {site}")

    def timed(fn):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
        torch.cuda.synchronize(device)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        for i in range(steps):
            evs[i][0].record(stream)
            fn(sptr)
            evs[i][1].record(stream)
        b.record(stream)
        torch.cuda.synchronize(device)
        return a.elapsed_time(b), sorted(x.elapsed_time(y) for x, y in evs)

    sampler = ClockSampler(device.index or 0)
    sampler.start()
    load_phase(lambda i: batch.run(sptr), device)
    grouped_ms, lat = timed(batch.run)
    clocks = with_window(sampler.stop())
    percall_ms, lat_pc = timed(batch.run_percall)
    st, site = batch.check_device()
    if st != wg.OK:
        raise RuntimeError(f"device wait gave up at site {site}")
    e2e = None
    if with_e2e:
        # inputs copied in from pinned host memory, outputs copied out
        hin = [torch.empty(x.shape, dtype=torch.float16).pin_memory() for x, _, _ in keep]
        hout = [torch.empty(y.shape, dtype=torch.float16).pin_memory() for _, _, y in keep]
        for h, (x, _, _) in zip(hin, keep):
            h.copy_(x.cpu())
        e_steps = max(3, min(steps, 10))
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        for _ in range(e_steps):
            for h, (x, _, _) in zip(hin, keep):
                x.copy_(h, non_blocking=True)
            batch.run(sptr)
            for h, (_, _, y) in zip(hout, keep):
                h.copy_(y, non_blocking=True)
            torch.cuda.synchronize(device)
        el = time.perf_counter() - t0
        e2e = {"value": flops * e_steps / el / 1e12, "unit": "TFLOP/s", "h2d_bytes_per_step": in_bytes,
               "d2h_bytes_per_step": out_bytes, "ms_per_step": el / e_steps * 1e3,
               "path": "pinned host copies of all 24 inputs/outputs around one grouped batch run"}
    out = {
        "workload": BATCH_WORKLOADS["cfg4"], "problems": [list(sh) for sh in shapes],
        "algo_bn": [batch.info(i) for i in range(len(shapes))], "total_gflop": flops / 1e9, "setup_s": setup_s,
        "grouped": {"tflops": flops * steps / (grouped_ms * 1e-3) / 1e12, "ms_per_step": grouped_ms / steps,
                    "launches": batch.launches(True), "p50_us": lat[len(lat) // 2] * 1e3,
                    "p99_us": lat[min(len(lat) - 1, int(0.99 * len(lat)))] * 1e3},
        "percall": {"tflops": flops * steps / (percall_ms * 1e-3) / 1e12, "ms_per_step": percall_ms / steps,
                    "launches": batch.launches(False), "p50_us": lat_pc[len(lat_pc) // 2] * 1e3,
                    "p99_us": lat_pc[min(len(lat_pc) - 1, int(0.99 * len(lat_pc)))] * 1e3,
                    "path": "each problem's own conv2d_fp16_ex launches, one problem after another on one stream"},
        "grouped_over_percall": percall_ms / grouped_ms,
        "steps": steps, "l2": f"working set {(in_bytes + out_bytes) / 2**30:.1f} GiB of inputs/outputs > L2",
        "e2e": e2e,
    }
    batch.destroy()
    del keep
    return out, clocks, flops


def batch_arm(args):
    """Batched workload as its own line (value = the grouped run)."""
    import torch
    rank, world, local = env_dist()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    wg = load_pkg()
    wg.lib()
    algo = ALGO_ARG[args.algo if args.algo != "ref" else "auto"]
    res, clocks, flops = batched_run(wg, torch, device, args.steps, args.warmup, algo, 99 + rank, not args.no_e2e)
    g = res["grouped"]
    line = {
        "metric": METRIC, "value": world * g["tflops"], "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": g["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f16", "data": "synthetic (seeded torch RNG)",
        "config": {"workload": res["workload"], "problems": res["problems"], "algo_bn": res["algo_bn"],
                   "total_gflop": res["total_gflop"], "accumulate": "fp32", "l2": res["l2"],
                   "setup_s": res["setup_s"]},
        "percall": res["percall"], "grouped_over_percall": res["grouped_over_percall"],
        "latency_us": {"p50": g["p50_us"], "p99": g["p99_us"], "percall_p50": res["percall"]["p50_us"]},
        "e2e": res["e2e"], "clocks": clocks, "roofline": None, "cpu_baseline": None,
        "gpu_launches": args.steps * g["launches"],
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def precision_arm(args):
    """F(4x3) precision study on the N=32, C=512, H=W=28, K=512 shape (the batch
    cut to --images images so the FP64 oracle finishes in seconds): for each
    input distribution (N(0,1); N(0,1) with 1% of entries x64), operand type
    (fp16, bf16), per-tile scaling (off, on) and F(4x3) point set, the max /
    mean relative error |y - ref| / max(|ref|, rms(ref)) against the FP64 direct
    convolution; F(2x3) rows for comparison."""
    import torch
    O = load_oracle()
    if not os.path.exists(O.LIB_PATH):
        O.build()
    wg = load_pkg()
    wg.lib()
    n, c, h, k = args.images, 512, 28, 512
    rows = []
    for dist in ("normal", "heavy"):
        x, wt = O.normal_inputs(2026, n, c, h, h, k, heavy=(dist == "heavy"))
        _, r64 = O.conv2d_direct(x, wt, nthreads=os.cpu_count() or 1)
        xt, wtt = torch.from_numpy(x).cuda(), torch.from_numpy(wt).cuda()
        for algo, points in ((0, 0), (0, 1), (1, 0)):
            for bf16 in (0, 1):
                for scaling in ((0, 1) if algo == 0 else (0,)):
                    opts = wg.default_options(algo=algo, operand_bf16=bf16, tile_scaling=scaling, f4_points=points)
                    y, op = wg.conv2d_torch(xt, wtt, 1, 1, opts)
                    torch.cuda.synchronize()
                    mx, mean, l2 = O.rel_errors(y.cpu().numpy(), r64)
                    rows.append({"input": dist, "algo": wg.ALGO_NAMES[algo],
                                 "points": ("reference 0,+-1,+-2" if points else "0,+-1,1/2,-2") if algo == 0 else "-",
                                 "operands": "bf16" if bf16 else "fp16", "tile_scaling": bool(scaling),
                                 "max_rel": mx, "mean_rel": mean, "l2_rel": l2})
                    op.destroy()
    print(json.dumps({"study": "F(4x3) precision vs FP64 direct convolution", "shape": [n, c, h, h, k],
                      "metric": "max/mean of |y-ref|/max(|ref|,rms(ref))", "rows": rows}), flush=True)
    return 0


def precision_line(wg, torch, device, images=2):
    """The precision study in compact form for the default line: `images`
    images of the N=32, C=512, H=W=28, K=512 shape, seeded N(0,1) inputs and
    the same with 1% of entries x64, filters N(0, 1/sqrt(9C)); max / mean
    relative error against an FP64 direct convolution (numpy, every output
    channel) for the default F(4x3) path with and without per-tile scaling,
    F(4x3) with bf16 operands and with the reference's points, and F(2x3)."""
    import numpy as np
    n, c, h, k = images, 512, 28, 512
    gen = torch.Generator().manual_seed(2027)
    w = torch.randn((k, c, 3, 3), generator=gen, dtype=torch.float64) / math.sqrt(9 * c)
    wt16 = w.half()
    w64 = wt16.double().numpy()
    rows = []
    t0 = time.time()
    for dist in ("normal", "heavy"):
        x = torch.randn((n, c, h, h), generator=gen, dtype=torch.float64)
        if dist == "heavy":
            x = torch.where(torch.rand(x.shape, generator=gen, dtype=torch.float64) < 0.01, x * 64, x)
        x16 = x.half()
        xp = np.zeros((n, c, h + 2, h + 2))
        xp[:, :, 1:h + 1, 1:h + 1] = x16.double().numpy()
        ref = np.zeros((n, k, h, h))
        for r in range(3):
            for s_ in range(3):
                ref += np.einsum("kc,nchw->nkhw", w64[:, :, r, s_], xp[:, :, r:r + h, s_:s_ + h], optimize=True)
        rms = math.sqrt(float(np.mean(ref * ref)))
        xd, wd = x16.to(device), wt16.to(device)
        for algo, bf16, scaling, points in ((0, 0, 0, 0), (0, 0, 1, 0), (0, 1, 0, 0), (0, 0, 0, 1), (1, 0, 0, 0)):
            opts = wg.default_options(algo=algo, operand_bf16=bf16, tile_scaling=scaling, f4_points=points)
            y, op = wg.conv2d_torch(xd, wd, 1, 1, opts)
            torch.cuda.synchronize()
            rel = np.abs(y.double().cpu().numpy() - ref) / np.maximum(np.abs(ref), rms)
            rows.append({"input": dist, "algo": wg.ALGO_NAMES[algo],
                         "points": ("reference 0,+-1,+-2" if points else "0,+-1,1/2,-2") if algo == 0 else "-",
                         "operands": "bf16" if bf16 else "fp16", "tile_scaling": bool(scaling),
                         "max": float(rel.max()), "mean": float(rel.mean())})
            op.destroy()
    return {"shape": [n, c, h, h, k], "against": "FP64 direct convolution, every output value",
            "measure": "|y - ref| / max(|ref|, rms(ref))", "bound": 2e-2, "rows": rows,
            "seconds": round(time.time() - t0, 1)}


def serve_layers(seed=20261203):
    """The 16 resident layers of the serving workload: (c, k, h) each."""
    import numpy as np
    rng = np.random.default_rng(seed)
    layers = []
    for _ in range(16):
        c = int(rng.choice([64, 128, 256, 512]))
        k = int(rng.choice([64, 128, 256, 512]))
        h = int(rng.choice([7, 14, 28, 56, 112]))
        layers.append((c, k, h))
    return layers, rng


def serving_run(wg, torch, device, count, rates, with_clocks=False):
    """One request trace through the continuous-batching server (6 slots, up
    to 16 requests per batch: the library's defaults) and through the plain per-call path (each
    request's own kernels queued on one stream at its arrival, no batching,
    no wait for earlier requests), same kernels and same arithmetic in both.
    Saturated (every request arriving at once) and at Poisson arrival rates
    given as multiples of the plain path's saturated capacity."""
    import numpy as np
    layers, rng = serve_layers()
    g = torch.Generator(device=device)
    g.manual_seed(7)
    bufs = []
    for c, k, h in layers:
        w = (torch.randn((k, c, 3, 3), generator=g, device=device) / math.sqrt(9 * c)).half()
        x = (torch.rand((64, c, h, h), generator=g, device=device) * 2 - 1).half()
        y = torch.empty((64, k, h, h), dtype=torch.float16, device=device)
        bufs.append((w, x, y))
    req_layer = rng.integers(0, 16, count).tolist()
    req_n = rng.integers(1, 65, count).tolist()
    flops = sum(direct_flops(req_n[i], layers[req_layer[i]][0], layers[req_layer[i]][2], layers[req_layer[i]][2],
                             layers[req_layer[i]][1]) for i in range(count))
    ins = [bufs[li][1].data_ptr() for li in req_layer]
    outs = [bufs[li][2].data_ptr() for li in req_layer]

    def make(served):
        srv = (wg.Server(slots=6, max_batch=16, hbm_budget_bytes=40 << 30) if served
               else wg.Server(per_request=1, hbm_budget_bytes=40 << 30))
        for (c, k, h), (w, _, _) in zip(layers, bufs):
            srv.add_layer(c, k, h, h, w.data_ptr())
        return srv

    def run(srv, rate):
        gaps = np.random.default_rng(11).exponential(1e6 / rate, count)
        arrivals = np.cumsum(gaps) - gaps[0]
        lat, wall = srv.replay(req_layer, req_n, arrivals.tolist(), ins, outs)
        lat = np.sort(np.array(lat))
        return {"rate_per_s": rate, "p50_us": float(lat[len(lat) // 2]), "p99_us": float(lat[int(0.99 * len(lat))]),
                "tflops": flops / (wall * 1e-6) / 1e12, "wall_s": wall * 1e-6}

    plain = make(False)
    served = make(True)
    # warm both (kernels, tensor maps), then measure the plain capacity:
    # every request arriving at once
    run(plain, 1e9)
    run(served, 1e9)
    sat_plain = run(plain, 1e9)
    capacity = count / sat_plain["wall_s"]
    sampler = ClockSampler(device.index or 0) if with_clocks else None
    if sampler:
        sampler.start()
    sweep = []
    for frac in rates:
        rate = frac * capacity
        sweep.append({"load_vs_plain_capacity": frac, "served": run(served, rate), "plain": run(plain, rate)})
    sat_served = run(served, 1e9)
    clocks = sampler.stop() if sampler else None
    st = served.stats()
    plain.destroy()
    served.destroy()
    out = {
        "workload": SERVE_WORKLOADS["cfg5"], "layers": [list(l) for l in layers], "requests": count,
        "total_gflop": flops / 1e9, "plain_capacity_req_per_s": capacity,
        "plain_path": "per-request kernels queued on one stream at arrival (server per_request mode)",
        "saturated": {"served": sat_served, "plain": sat_plain,
                      "served_over_plain": sat_served["tflops"] / sat_plain["tflops"]},
        "sweep": sweep, "server_stats": st,
    }
    del bufs
    return out, clocks


def serve_arm(args):
    """Serving workload as its own line (value = the saturated served run)."""
    import torch
    rank, world, local = env_dist()
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    wg = load_pkg()
    wg.lib()
    res, clocks = serving_run(wg, torch, device, args.requests, args.rates, with_clocks=True)
    sat = res["saturated"]["served"]
    line = {
        "metric": METRIC, "value": world * sat["tflops"], "unit": "TFLOP/s", "n_gpus": world,
        "steps": args.requests, "warmup": args.requests, "ms_per_step": sat["wall_s"] * 1e3 / args.requests,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f16",
        "data": "synthetic (seeded)",
        "config": {"workload": res["workload"], "layers": res["layers"], "requests": args.requests,
                   "total_gflop": res["total_gflop"], "plain_capacity_req_per_s": res["plain_capacity_req_per_s"]},
        "saturated": res["saturated"], "sweep": res["sweep"], "server_stats": res["server_stats"],
        "clocks": clocks, "roofline": None, "cpu_baseline": None, "e2e": None, "gpu_launches": None,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    return 0


def time_cudnn(torch, x, w, steps, warmup):
    """cuDNN through torch's conv2d (fp16, NCHW, pad 1), device time per call."""
    import torch.nn.functional as F
    torch.backends.cudnn.benchmark = True
    for _ in range(max(3, warmup)):
        F.conv2d(x, w, padding=1)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(steps):
        F.conv2d(x, w, padding=1)
    b.record()
    torch.cuda.synchronize()
    return a.elapsed_time(b) / steps


def suite_arm(args):
    """The reference's contest shapes (its pre.sh and final.sh) through the
    drop-in API, with the reference's selection and with the autotuner, beside
    cuDNN and the reference's published DCU latencies."""
    import torch
    wg = load_pkg()
    wg.lib()
    rows = []
    names = [f"pre{i}" for i in range(1, 7)] + [f"final{i}" for i in range(1, 7)] + ["cfg1", "cfg2", "cfg3"]
    for name in names:
        n, c, h, w, k, xd, wd, desc = WORKLOADS[name]
        x, wt = make_inputs(torch, name, torch.device("cuda"), 77)
        y = torch.empty((n, k, h, w), dtype=torch.float16, device="cuda")
        fl = direct_flops(n, c, h, w, k)
        row = {"shape": name, "n": n, "c": c, "h": h, "w": w, "k": k}
        for label, algo in (("reference_selection", -1), ("auto", 3)):
            op = wg.Conv2d(wg.make_problem(x.data_ptr(), wt.data_ptr(), y.data_ptr(), n, c, h, w, k),
                           wg.default_options(algo=algo))
            s = torch.cuda.current_stream().cuda_stream
            for _ in range(3):
                op(s)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(args.steps):
                op(s)
            b.record()
            torch.cuda.synchronize()
            us = a.elapsed_time(b) / args.steps * 1e3
            row[label] = {"algo": wg.ALGO_NAMES[op.algo], "us": us, "tflops": fl / (us * 1e-6) / 1e12}
            op.destroy()
        us = time_cudnn(torch, x, wt, args.steps, args.warmup) * 1e3
        row["cudnn"] = {"us": us, "tflops": fl / (us * 1e-6) / 1e12}
        if name in PUBLISHED_US:
            row["reference_dcu_us"] = PUBLISHED_US[name]
        rows.append(row)
    print(json.dumps({"suite": "contest shapes, 3x3 pad 1 stride 1 fp16", "steps": args.steps, "rows": rows}),
          flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS) + sorted(BATCH_WORKLOADS) + sorted(SERVE_WORKLOADS),
                    default="cfg2")
    ap.add_argument("--requests", type=int, default=20000, help="requests of the serving trace")
    ap.add_argument("--rates", type=float, nargs="*", default=[0.5, 0.9, 1.2],
                    help="arrival rates of the serving sweep, as multiples of the plain capacity")
    ap.add_argument("--algo", choices=sorted(ALGO_ARG), default="auto")
    ap.add_argument("--gemm-bn", type=int, default=0)
    ap.add_argument("--l2-chunk", type=int, default=None)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--precision", action="store_true", help="F(4x3) precision study instead of timing")
    ap.add_argument("--suite", action="store_true", help="contest shapes through the drop-in API, with cuDNN")
    ap.add_argument("--no-cudnn", action="store_true", help="skip the cuDNN (torch conv2d) comparison")
    ap.add_argument("--no-serving", action="store_true",
                    help="skip the batched (24 uneven problems) and served (request trace) comparisons of the default line")
    ap.add_argument("--line-requests", type=int, default=2000, help="requests of the default line's serving trace")
    ap.add_argument("--nhwc", action="store_true", help="channels-last input and output tensors")
    ap.add_argument("--m-fp32", action="store_true", help="F(4x3): store the GEMM result M in fp32 instead of 24 bits")
    ap.add_argument("--images", type=int, default=4, help="images of the precision study")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the default line's precision record (2 images of N=32 C=512 28x28 K=512)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)
    if args.precision:
        return precision_arm(args)
    if args.suite:
        return suite_arm(args)
    if args.workload in SERVE_WORKLOADS:
        return serve_arm(args)
    if args.workload in BATCH_WORKLOADS:
        return batch_arm(args)
    return our_arm(args)


if __name__ == "__main__":
    sys.exit(main())

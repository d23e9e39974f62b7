#!/usr/bin/env python3
"""Encrypted predictions/s of the party-B scoring step (cloud_compute_score,
eval/idash.cpp:763-848) on GB300.

One step = one pass of the scoring step over one batch: every output
ciphertext of the model computed once.  Default workload (full scale, the
reference's TRLWE-packed layout): 1,000 individuals packed in one region per
TRLWE (N = 1024), 16,184 tag SNPs (48,552 input TRLWE), 80,882 targets x 3
outputs (242,646 output TRLWE), 5 nearest-tag neighbours, coefficients
uniform in [-8192, 8191]; synthetic seeded data.

  value        predictions/s with inputs and model resident in HBM (CUDA
               events on the launching stream; inputs 0.4 GB > L2, outputs 2 GB)
  e2e          the same through idash_score_trlwe_host with page-locked host
               buffers: every step copies the inputs in and the outputs out
  roofline     the scoring kernel against the measured HBM copy bandwidth
  cpu_baseline the oracle's restatement of the reference loop on the host cores
  forms        the other configurations and layouts, each with its own bound
               and a CPU timing of the oracle beside it (sampled where a full
               pass is too slow for the host, and labelled so)

--impl reference times that CPU restatement alone (all host threads) on the
same workload and prints the same line with impl=reference; it builds the
workload from the oracle alone (no part of the GPU library is loaded).
Multi-GPU (torchrun): each rank scores its own batch of the same size
(weak scaling, no collective on the data path); max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

WORKLOADS = {
    "trlwe_full": dict(n_indiv=1000, n_tags=16184, n_targets=80882, neighbours=5,
                       desc="full scale, TRLWE-packed (reference layout): 1,000 individuals, 16,184 tags, "
                            "80,882 targets x 3 outputs, 5 neighbours, N=1024, NUM_REGIONS=1"),
    "trlwe_prof": dict(n_indiv=1000, n_tags=8000, n_targets=40000, neighbours=5,
                       desc="profiling size, TRLWE-packed: 1,000 individuals, 8,000 tags, 40,000 targets x 3 outputs, "
                            "5 neighbours, NUM_REGIONS=1 (inputs 197 MB > L2)"),
    "trlwe_n10": dict(n_indiv=1000, n_tags=16184, n_targets=80882, neighbours=10,
                      desc="full scale, TRLWE-packed, 10 neighbours (the served model): 1,000 individuals, "
                           "16,184 tags, 80,882 targets x 3 outputs, N=1024, NUM_REGIONS=1"),
    "trlwe_r10": dict(n_indiv=100, n_tags=500, n_targets=2000, neighbours=5,
                      desc="CPU-runnable size, TRLWE-packed: 100 individuals (NUM_REGIONS=10, REGION_SIZE=102), "
                           "500 tags, 2,000 targets x 3 outputs, 5 neighbours"),
}
METRIC = "encrypted predictions/s (indiv x target x 3)"
UNIT = "predictions/s"
# The reference's one published run of this step: 1,004 individuals x 80,882
# targets x 3 in 3.06433 s of "fhe wall time" on a 4-thread laptop
# (README.md:220-245), i.e. about 79.5 M predictions/s.
PUBLISHED_PREDICTIONS_PER_S = 1004 * 80882 * 3 / 3.06433
KERNEL_NAMES = {0: "window", 1: "direct (plain)", 2: "pipe", 3: "ws (warp-specialised, IMAD)",
                4: "tc (tensor cores, exact fp16 digit products)"}
# 32-bit integer multiply-adds per second measured on this GB300 (one-off
# throughput probe, profiles/device_limits.txt)
IMAD_PEAK = 20.07e12
CONSTANT = 0xFFFFFFFF


def sig(x, n=4):
    """x with floats rounded to n significant digits (recursively)."""
    if isinstance(x, float):
        return float(f"{x:.{n}g}")
    if isinstance(x, dict):
        return {k: sig(v, n) for k, v in x.items()}
    if isinstance(x, (list, tuple)):
        return [sig(v, n) for v in x]
    return x


class timed_range:
    """NVTX push/pop range 'timed' around a timed region, so that a profiler
    can be limited to it (ncu --nvtx --nvtx-include timed/)."""

    def __enter__(self):
        import torch
        torch.cuda.nvtx.range_push("timed")

    def __exit__(self, *exc):
        import torch
        torch.cuda.nvtx.range_pop()


def peaks():
    """Measured HBM copy bandwidth (GB/s) and dense bf16 tensor rate
    (TFLOP/s, burst) from MEASURED_PEAKS.json, else the machine's fallback."""
    try:
        p = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return {"hbm": float(p["hbm_gbs"]), "bf16": float(p["bf16_tflops"]), "source": "measured"}
    except Exception:
        return {"hbm": 6800.0, "bf16": 1900.0, "source": "fallback"}


def profiled_traffic(name: str):
    """dram bytes per launch recorded from an ncu capture in profiles/<name>."""
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            if line.startswith("traffic_bytes_per_launch:"):
                return float(line.split(":", 1)[1].split()[0])
    except OSError:
        pass
    return None


def hbm_roofline(alg_bytes, seconds):
    p = peaks()
    achieved = alg_bytes / seconds / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": p["hbm"], "unit": "GB/s", "frac": achieved / p["hbm"],
            "peak_source": p["source"]}


def compute_roofline(kind, useful_macs, dense_macs, alg_bytes, seconds):
    """The bound of an accumulate kernel that is not HBM-bound: the IMAD
    kernels against the measured IMAD rate (useful multiply-adds), the
    tensor-core kernel against the measured dense fp16/bf16 tensor rate
    (digit multiply-adds it executes, padding included); the HBM fraction of
    the algorithmic bytes beside it."""
    p = peaks()
    hbm = hbm_roofline(alg_bytes, seconds)
    if kind == 4:
        achieved = dense_macs / seconds / 1e12
        peak = p["bf16"] / 2
        out = {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "T MAC/s", "frac": achieved / peak}
    else:
        achieved = useful_macs / seconds / 1e12
        out = {"bound": "imad", "achieved": achieved, "peak": IMAD_PEAK / 1e12, "unit": "T MAC/s",
               "frac": achieved / (IMAD_PEAK / 1e12)}
    out["useful_mac_per_s"] = useful_macs / seconds
    out["hbm_frac"] = hbm["frac"]
    out["hbm_achieved_gbs"] = hbm["achieved"]
    return out


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.samples = []
        self.proc = None
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 9:
                self.samples.append((time.time(), parts))

    def stop(self):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self, t0: float, t1: float):
        sel = [s for t, s in self.samples if t0 - 0.25 <= t <= t1 + 0.25]
        if not sel and self.samples:
            mid = (t0 + t1) / 2
            sel = [min(self.samples, key=lambda ts: abs(ts[0] - mid))[1]]
        if not sel:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        mhz = sorted(float(s[1]) for s in sel if s[1].replace(".", "").isdigit())
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in sel for i in range(4) if s[5 + i].lower().startswith("active")})
        return {"sm_mhz": mhz[len(mhz) // 2] if mhz else None,
                "sm_max_mhz": float(sel[0][2]) if sel[0][2].replace(".", "").isdigit() else None,
                "reasons": reasons, "samples": len(sel)}



def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", str(rank)))
    return rank, world, local


def max_over_ranks(x: float) -> float:
    """The largest x over the process group (x itself without one): a
    multi-GPU timing is the slowest rank's.  NCCL reduces on the device, gloo
    on the host."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return x
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if dist.get_backend() == "nccl" else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload_spec(name):
    spec = dict(WORKLOADS[name])
    regions = max(1, 1024 // spec["n_indiv"])
    spec.update(regions=regions, region_size=1024 // regions, num_samples=spec["n_indiv"],
                n_rows=(3 * spec["n_tags"] + regions - 1) // regions)
    return spec


def config_of(spec, world):
    """The workload as both arms print it (the same keys and values)."""
    in_bytes, out_bytes = spec["n_rows"] * 8192, 3 * spec["n_targets"] * 8192
    return {"workload": spec["desc"], "individuals": spec["n_indiv"], "targets": spec["n_targets"],
            "tags": spec["n_tags"], "neighbours": spec["neighbours"], "outputs": 3 * spec["n_targets"],
            "input_rows": spec["n_rows"], "num_regions": spec["regions"], "region_size": spec["region_size"],
            "l2": f"inputs {in_bytes / 1e9:.2f} GB and outputs {out_bytes / 1e9:.2f} GB vs the 129 MB L2",
            "parallelism": f"{world} independent batch(es)"}


def cores():
    return os.cpu_count() or 1


def repeat_timed(fn, min_seconds, max_reps=1000):
    """(reps, seconds): fn() run until min_seconds have passed."""
    reps, t0 = 0, time.perf_counter()
    while True:
        fn()
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or reps >= max_reps:
            return reps, el


def cpu_trlwe(ptr, feat, coef, rows, spec, min_seconds):
    """The oracle's restatement of the reference loop (OpenMP over outputs,
    eval/idash.cpp:779-842) on all host cores, full workload per rep."""
    import pyoracle
    preds = spec["n_indiv"] * spec["n_targets"] * 3
    reps, el = repeat_timed(lambda: pyoracle.trlwe_score(ptr, feat, coef, rows, spec["num_samples"], spec["regions"],
                                                         spec["region_size"], n_threads=cores()), min_seconds)
    return {"value": preds * reps / el, "unit": UNIT, "cores": cores(), "kind": "port",
            "sample": f"{reps} full passes ({el:.1f} s), oracle/oracle.c restatement of eval/idash.cpp:779-842, "
                      f"OpenMP {cores()} threads"}


def run_reference(args):
    """The reference loop on the host cores: the oracle's restatement of
    eval/idash.cpp:779-842 (the reference binary needs the absent TFHE
    library).  The workload comes from the oracle's own restatement of the
    synthetic generator, so nothing of the GPU library is loaded."""
    import numpy as np
    import pyoracle
    rank, world, _ = dist_env()
    if rank != 0:
        return
    spec = workload_spec(args.workload)
    ptr, feat, coef, _, _ = pyoracle.synth_model(args.seed, spec["n_tags"], spec["n_targets"],
                                                 neighbours=spec["neighbours"])
    rng = np.random.default_rng(args.seed)
    rows = rng.integers(0, 2 ** 32, size=(spec["n_rows"], 2048), dtype=np.uint64).astype(np.uint32).view(np.int32)
    steps = args.steps if args.steps_given else 3
    # one full pass per step, or, when K full passes would take more than
    # about two minutes, the same leading share of the targets in every step
    # (a bounded sample; the rate is per prediction either way)
    t0 = time.perf_counter()
    pyoracle.trlwe_score(ptr, feat, coef, rows, spec["num_samples"], spec["regions"], spec["region_size"],
                         n_threads=cores())
    full_s = time.perf_counter() - t0
    share = min(1.0, 120.0 / max(steps * full_s, 1e-9))
    n_tg = max(1, int(spec["n_targets"] * share))
    sub_ptr = ptr[:3 * n_tg + 1]
    preds = spec["n_indiv"] * n_tg * 3
    run = lambda: pyoracle.trlwe_score(sub_ptr, feat[:int(sub_ptr[-1])], coef[:int(sub_ptr[-1])], rows,
                                       spec["num_samples"], spec["regions"], spec["region_size"], n_threads=cores())
    for _ in range(args.warmup):
        run()
    t0 = time.perf_counter()
    for _ in range(steps):
        run()
    el = time.perf_counter() - t0
    value = preds * steps / el
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": el / steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": value / PUBLISHED_PREDICTIONS_PER_S if args.workload == "trlwe_full" else None,
            "dtype": "int32 (Z/2^32)", "data": "synthetic (seeded)", "impl": "reference",
            "config": config_of(spec, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores(), "kind": "port",
                             "sample": (f"{steps} full passes" if n_tg == spec["n_targets"] else
                                        f"{steps} passes over the first {n_tg} of {spec['n_targets']} targets") +
                                       "; oracle/oracle.c restatement of eval/idash.cpp:779-842 "
                                       f"(the reference's TFHE dependency is absent, so its cloud binary cannot be "
                                       f"built on this host)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(sig(line)), flush=True)


def time_on_stream(ctx, fn, steps):
    """ms per call of fn(), CUDA events on the context's stream."""
    import torch
    stream = torch.cuda.ExternalStream(ctx.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ctx.sync()
    e0.record(stream)
    with timed_range():
        for _ in range(steps):
            fn()
    e1.record(stream)
    e1.synchronize()
    ctx.sync()
    return e0.elapsed_time(e1) / steps


def trlwe_alg_bytes(info, n_out):
    """Each distinct input TRLWE read once, each output TRLWE written once,
    the model's CSR (4 B feature + 4 B coefficient per term, 4 B bias + 4 B
    row pointer per output)."""
    return info["algorithmic_in_rows"] * 8192 + n_out * 8192 + info["n_terms"] * 8 + n_out * 8


def section_plain(ctx, w, spec, d_in, d_out, steps):
    """The plain per-output kernel (k_score_direct) on the same workload."""
    from idash2019_2_gb300 import gpu
    ctx.set_option("kernel", 1)
    try:
        m = gpu.TrlweModel(ctx, w.model, spec["n_rows"], spec["num_samples"], spec["regions"], spec["region_size"])
        lay = gpu.DENSE_TRLWE
        for _ in range(3):
            m.score_device(d_in.ptr, lay, d_out.ptr, lay)
        ms = time_on_stream(ctx, lambda: m.score_device(d_in.ptr, lay, d_out.ptr, lay), steps)
        info = m.info()
        m.free()
    finally:
        ctx.set_option("kernel", 0)
    preds = spec["n_indiv"] * spec["n_targets"] * 3
    return {"value": preds / (ms / 1e3), "ms_per_step": ms,
            "roofline": hbm_roofline(trlwe_alg_bytes(info, 3 * spec["n_targets"]), ms / 1e3)}


def section_kinds(ctx, w, spec, d_in, d_out, steps):
    """Each batched kernel kind on the headline workload, autotuned within its
    kind (slice width, CTAs per SM, ring depth): ms per pass."""
    from idash2019_2_gb300 import gpu
    out = {}
    lay = gpu.DENSE_TRLWE
    for option, name in ((2, "window"), (3, "pipe"), (4, "ws"), (5, "tc")):
        ctx.set_option("kernel", option)
        try:
            m = gpu.TrlweModel(ctx, w.model, spec["n_rows"], spec["num_samples"], spec["regions"],
                               spec["region_size"])
            for _ in range(3):
                m.score_device(d_in.ptr, lay, d_out.ptr, lay)
            out[name] = time_on_stream(ctx, lambda: m.score_device(d_in.ptr, lay, d_out.ptr, lay), steps)
            m.free()
        finally:
            ctx.set_option("kernel", 0)
    return out


def copy_d2h(ctx, host_ptr, dev_ptr, nbytes):
    import ctypes as C
    ctx.check(ctx.lib.idash_copy_d2h(ctx.h, C.c_void_p(host_ptr), C.c_void_p(dev_ptr), nbytes))


def copy_h2d(ctx, dev_ptr, host_ptr, nbytes):
    import ctypes as C
    ctx.check(ctx.lib.idash_copy_h2d(ctx.h, C.c_void_p(dev_ptr), C.c_void_p(host_ptr), nbytes))


def section_config1(ctx, seed):
    """Configuration 1 (100 individuals, 500 tags, 2,000 targets x 3, 5
    neighbours) in both layouts: TRLWE-packed as the reference packs 100
    individuals (NUM_REGIONS 10, REGION_SIZE 102) and per-individual LWE
    (n = 1024).  Each: device-resident value, e2e from page-locked host
    buffers (inputs copied in and outputs copied out every step), roofline,
    and the oracle on all host cores over the whole workload."""
    import numpy as np
    import pyoracle
    from idash2019_2_gb300 import gpu
    out = {}
    spec = workload_spec("trlwe_r10")
    preds = spec["n_indiv"] * spec["n_targets"] * 3
    w = gpu.synth_model(seed, spec["n_tags"], spec["n_targets"], neighbours=5)
    csr = w.model
    # TRLWE-packed
    params = gpu.TrlweParams(1024, 1, spec["num_samples"], spec["regions"], spec["region_size"], 1 << 18, 42)
    m = gpu.TrlweModel(ctx, csr, spec["n_rows"], spec["num_samples"], spec["regions"], spec["region_size"])
    d_in, d_out = ctx.device_alloc(spec["n_rows"] * 8192), ctx.device_alloc(csr.n_out * 8192)
    gpu.synth_trlwe_device(ctx, seed, params, spec["n_tags"], d_in.ptr, gpu.DENSE_TRLWE)
    lay = gpu.DENSE_TRLWE
    run = lambda: m.score_device(d_in.ptr, lay, d_out.ptr, lay)
    for _ in range(3):
        run()
    ms = time_on_stream(ctx, run, 200)
    info = m.info()
    h_in, h_out = ctx.host_alloc(spec["n_rows"] * 8192), ctx.host_alloc(csr.n_out * 8192)
    h_in.array[:] = d_in.download()
    m.score_host(h_in.ptr, lay, spec["n_rows"], h_out.ptr, lay)
    reps, el = repeat_timed(lambda: m.score_host(h_in.ptr, lay, spec["n_rows"], h_out.ptr, lay), 0.5)
    rows = np.frombuffer(h_in.array, np.int32).reshape(spec["n_rows"], 2048).copy()
    out["trlwe"] = {"value": preds / (ms / 1e3), "ms_per_step": ms, "kernel": KERNEL_NAMES.get(info["kernel"]),
                    "roofline": hbm_roofline(trlwe_alg_bytes(info, csr.n_out), ms / 1e3),
                    "e2e": {"value": preds * reps / el, "unit": UNIT, "ms_per_step": el / reps * 1e3,
                            "h2d_bytes_per_step": spec["n_rows"] * 8192, "d2h_bytes_per_step": csr.n_out * 8192},
                    "cpu_baseline": cpu_trlwe(csr.term_ptr, csr.term_feat, csr.term_coef, rows, spec, 3.0)}
    for b in (d_in, d_out, h_in, h_out):
        b.free()
    m.free()
    # per-individual LWE
    n_indiv, n = 100, 1024
    n_feat = 3 * spec["n_tags"]
    stride = gpu.lwe_row_words(n_indiv, n)
    L = n_indiv * (n + 1)
    lm = gpu.LweModel(ctx, csr, n_feat, n_indiv, n)
    d_in, d_out = ctx.device_alloc(n_feat * stride * 4), ctx.device_alloc(csr.n_out * stride * 4)
    gpu.synth_lwe_device(ctx, seed, n, n_indiv, n_feat, d_in.ptr, stride)
    run = lambda: lm.score_device(n_indiv, d_in.ptr, stride, 0, csr.n_out, d_out.ptr, stride)
    run()
    ms = time_on_stream(ctx, run, 10)
    info = lm.info()
    h_in, h_out = ctx.host_alloc(n_feat * stride * 4), ctx.host_alloc(csr.n_out * stride * 4)
    h_in.array[:] = d_in.download()

    def e2e_step():
        copy_h2d(ctx, d_in.ptr, h_in.ptr, n_feat * stride * 4)
        run()
        copy_d2h(ctx, h_out.ptr, d_out.ptr, csr.n_out * stride * 4)

    e2e_step()
    reps, el = repeat_timed(e2e_step, 0.5)
    rows = np.frombuffer(h_in.array, np.int32).reshape(n_feat, stride).copy()
    creps, cel = repeat_timed(lambda: pyoracle.lwe_score(csr.term_ptr, csr.term_feat, csr.term_coef, rows, n_indiv,
                                                         0, csr.n_out, n=n, n_threads=cores()), 3.0, 20)
    alg = info["algorithmic_in_rows"] * L * 4 + csr.n_out * L * 4 + info["n_terms"] * 8 + csr.n_out * 8
    useful = float(np.count_nonzero(csr.term_feat != CONSTANT)) * L
    dense = 7.0 * 128 * info["dense_k"] * L
    out["lwe"] = {"value": preds / (ms / 1e3), "ms_per_step": ms, "kernel": KERNEL_NAMES.get(info["kernel"]),
                  "roofline": hbm_roofline(alg, ms / 1e3),
                  "compute": compute_roofline(info["kernel"], useful, dense, alg, ms / 1e3),
                  "e2e": {"value": preds * reps / el, "unit": UNIT, "ms_per_step": el / reps * 1e3,
                          "h2d_bytes_per_step": n_feat * stride * 4, "d2h_bytes_per_step": csr.n_out * stride * 4},
                  "cpu_baseline": {"value": preds * creps / cel, "unit": UNIT, "cores": cores(), "kind": "port",
                                   "sample": f"{creps} full passes ({cel:.1f} s), oracle LWE restatement, "
                                             f"OpenMP {cores()} threads"}}
    for b in (d_in, d_out, h_in, h_out):
        b.free()
    lm.free()
    return out


def section_lwe(ctx, seed, n_indiv, n_tags, n_targets, neighbours=5, choices=None, passes=2, chunk=2048,
                cpu_outputs=48):
    """Per-individual LWE form: inputs resident (n_indiv LWE samples of n=1024
    per feature row), outputs produced range by range into a 2-slot HBM ring
    (the full output does not fit in HBM).  The CPU baseline times the oracle
    on cpu_outputs outputs spread over the model (their input rows copied
    back from the device) and scales to predictions/s."""
    import numpy as np
    import pyoracle
    from idash2019_2_gb300 import gpu
    w = gpu.synth_model(seed, n_tags, n_targets, neighbours=neighbours, choices=choices)
    csr = w.model
    n_feat = 3 * n_tags
    stride = gpu.lwe_row_words(n_indiv)
    L = n_indiv * 1025
    d_in = ctx.device_alloc(n_feat * stride * 4)
    gpu.synth_lwe_device(ctx, seed, 1024, n_indiv, n_feat, d_in.ptr, stride)
    m = gpu.LweModel(ctx, csr, n_feat, n_indiv)
    ring = [ctx.device_alloc(chunk * stride * 4) for _ in range(2)]
    ranges = [(lo, min(lo + chunk, m.n_out)) for lo in range(0, m.n_out, chunk)]

    def one_pass():
        for c, (lo, hi) in enumerate(ranges):
            m.score_device(n_indiv, d_in.ptr, stride, lo, hi, ring[c % 2].ptr, stride)

    t0 = time.perf_counter()
    one_pass()  # the first call autotunes
    ctx.sync()
    first_s = time.perf_counter() - t0
    launches0 = ctx.stats()["kernel_launches"]
    ms = time_on_stream(ctx, one_pass, passes)
    launches = (ctx.stats()["kernel_launches"] - launches0) // passes
    info = m.info()
    preds = n_indiv * n_targets * 3
    alg = info["algorithmic_in_rows"] * L * 4 + m.n_out * L * 4 + info["n_terms"] * 8 + m.n_out * 8
    useful = float(np.count_nonzero(csr.term_feat != CONSTANT)) * L
    dense = 7.0 * 128 * info["dense_k"] * L
    # CPU baseline on a sample: 4 runs of cpu_outputs / 4 outputs
    spent, done = 0.0, 0
    for lo in np.linspace(0, m.n_out - cpu_outputs // 4, 4).astype(int):
        hi = int(lo) + cpu_outputs // 4
        a, b = int(csr.term_ptr[lo]), int(csr.term_ptr[hi])
        f = csr.term_feat[a:b]
        real = f != CONSTANT
        f0, f1 = int(f[real].min()), int(f[real].max()) + 1
        rows = d_in.download(nbytes=(f1 - f0) * stride * 4, offset=f0 * stride * 4, dtype=np.int32).reshape(f1 - f0,
                                                                                                          stride)
        feat = f.copy()
        feat[real] -= f0
        ptr = (csr.term_ptr[lo:hi + 1] - a).astype(np.uint64)
        t1 = time.perf_counter()
        pyoracle.lwe_score(ptr, feat, csr.term_coef[a:b], rows, n_indiv, 0, hi - lo, n_threads=cores())
        spent += time.perf_counter() - t1
        done += hi - lo
    out = {"value": preds / (ms / 1e3), "ms_per_step": ms, "kernel": KERNEL_NAMES.get(info["kernel"]),
           "slice_words": info["slice_words"], "launches_per_step": launches, "first_pass_s": first_s,
           "roofline": compute_roofline(info["kernel"], useful, dense, alg, ms / 1e3),
           "cpu_baseline": {"value": done * n_indiv / spent, "unit": UNIT, "cores": cores(), "kind": "port",
                            "sample": f"{done} of {m.n_out} outputs in 4 ranges, {spent:.1f} s, oracle LWE "
                                      f"restatement, scaled to predictions/s"}}
    for b in ring:
        b.free()
    d_in.free()
    m.free()
    return out


def section_intpoly(ctx, seed, passes=5, scale=1, cpu_outputs=24):
    """Integer-polynomial x TRLWE product at full scale: 48,552 input TRLWE
    (16,184 tags x 3), 242,646 outputs (80,882 targets x 3), 20 neighbours
    (60 dense int16 weight polynomials per output, |w| <= 8192), one block of
    1,024 individuals per TRLWE.  Exact (two-prime NTT + CRT).  scale > 1
    divides the tag and target counts (profiling size).  The CPU baseline is
    the oracle's schoolbook product on cpu_outputs outputs, scaled."""
    import numpy as np
    import pyoracle
    from idash2019_2_gb300 import gpu
    n_tags, n_targets = 16184 // scale, 80882 // scale
    w = gpu.synth_model(seed, n_tags, n_targets, neighbours=20)
    csr = w.model
    const = csr.term_feat == CONSTANT
    owner = np.repeat(np.arange(csr.n_out), np.diff(csr.term_ptr.astype(np.int64)))
    counts = np.bincount(owner[~const], minlength=csr.n_out)
    ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint64)
    feat = csr.term_feat[~const]
    bias = np.zeros(csr.n_out, np.int32)
    bias[owner[const]] = csr.term_coef[const]
    icsr = gpu.CSRModel(ptr, feat, np.zeros(len(feat), np.int32))
    n_terms, n_rows = len(feat), 3 * n_tags
    d_poly = ctx.device_alloc(n_terms * 1024 * 2)
    gpu.synth_int16_device(ctx, seed, n_terms * 1024, 8192, d_poly.ptr)
    t0 = time.perf_counter()
    m = gpu.IntpolyModel(ctx, icsr, d_poly.ptr, n_rows, 1024, 1024, bias=bias, poly_on_device=True)
    build_s = time.perf_counter() - t0
    polys = d_poly.download(nbytes=int(ptr[cpu_outputs]) * 2048, dtype=np.int16).reshape(-1, 1024)
    d_poly.free()
    params = gpu.TrlweParams(1024, 1, 1024, 1, 1024, 1 << 18, 42)
    d_in = ctx.device_alloc(n_rows * 8192)
    gpu.synth_trlwe_device(ctx, seed, params, n_tags, d_in.ptr, gpu.DENSE_TRLWE)
    d_out = ctx.device_alloc(csr.n_out * 8192)
    run = lambda: m.score_device(d_in.ptr, gpu.DENSE_TRLWE, 0, csr.n_out, d_out.ptr, gpu.DENSE_TRLWE)
    run()
    ms = time_on_stream(ctx, run, passes)
    # The stored-form trade: resident transformed weights (2 primes x 1,024
    # words = 8 KiB a term, read every pass) against int16 weights (2 KiB a
    # term) transformed on every pass.  The transform's own time bounds what
    # any pass that starts from int16 weights costs above the scoring.
    d_w16 = ctx.device_alloc(n_terms * 1024 * 2)
    gpu.synth_int16_device(ctx, seed, n_terms * 1024, 8192, d_w16.ptr)  # the same weights again
    transform = lambda: m.set_weights(d_w16.ptr)
    transform()
    transform_ms = time_on_stream(ctx, transform, passes)
    alt_ms = time_on_stream(ctx, lambda: (transform(), run()), passes)
    d_w16.free()
    weights = {"resident_transform": {"bytes_per_term": 8192, "ms_per_step": ms},
               "int16_transformed_each_pass": {"bytes_per_term": 2048, "ms_per_step": alt_ms,
                                               "transform_ms": transform_ms,
                                               "transform_hbm_frac": hbm_roofline(n_terms * (2048 + 8192),
                                                                                  transform_ms / 1e3)["frac"]},
               "kept": "resident_transform" if ms <= alt_ms else "int16_transformed_each_pass"}
    rows = d_in.download(dtype=np.int32).reshape(n_rows, 2048)
    t1 = time.perf_counter()
    pyoracle.intpoly_score(ptr[:cpu_outputs + 1], feat[:int(ptr[cpu_outputs])], polys, bias[:cpu_outputs], rows,
                           1024, 1024, 0, cpu_outputs, n_threads=cores())
    cpu_s = time.perf_counter() - t1
    # The configuration's own algorithmic bytes: int16 weights (2 KiB per
    # term), input rows in, output rows out.  This implementation keeps the
    # weights resident NTT-transformed (2 primes x 1,024 words = 8 KiB per
    # term) and also writes and reads the inputs' transforms: its own
    # compulsory bytes are larger by the ratio below.
    alg = n_terms * 1024 * 2 + n_rows * 8192 + csr.n_out * 8192
    traffic = n_terms * 2 * 1024 * 4 + n_rows * 8192 + 2 * n_rows * 4 * 1024 * 4 + csr.n_out * 8192
    out = {"value": csr.n_out * 1024 / (ms / 1e3), "ms_per_step": ms, "outputs_per_s": csr.n_out / (ms / 1e3),
           "terms": n_terms, "model_build_s": build_s,
           "schoolbook_mac_per_s": n_terms * 2 * 1024 * 1024 / (ms / 1e3),
           "weights": weights,
           "roofline": hbm_roofline(alg, ms / 1e3),
           "representation": {"bytes_per_step": traffic, "over_config_bytes": traffic / alg,
                              "frac": hbm_roofline(traffic, ms / 1e3)["frac"]},
           "cpu_baseline": {"value": cpu_outputs * 1024 / cpu_s, "unit": UNIT, "cores": cores(), "kind": "port",
                            "sample": f"{cpu_outputs} of {csr.n_out} outputs ({cpu_s:.1f} s), oracle schoolbook "
                                      f"negacyclic product, scaled to predictions/s"}}
    for b in (d_in, d_out):
        b.free()
    m.free()
    return out


def section_serving(ctx, seed, n_requests=10000, budget=150 << 30, inflight=16, cpu_requests=6, e2e_requests=200,
                    lwe_requests=12):
    """Configuration 5: an online server (idash_server_*) over one resident
    model with 10 neighbours and a 150 GB HBM admission budget; requests of
    individuals ~ U[1, 2000] and a contiguous target range of length
    ~ U[1000, 80882].
      trlwe      10,000 requests arriving as a Poisson stream at 0.8 x the
                 measured capacity (TRLWE-packed, 1,024 individuals per block;
                 ciphertexts generated on the device, outputs digested):
                 throughput, p50/p99 latency, HBM roofline of the bytes the
                 requests move, CPU baseline on a sample of requests;
      e2e        e2e_requests requests with their ciphertexts in page-locked
                 host memory and their outputs copied back, four in flight
                 from the client's side (a closed loop);
      lwe        lwe_requests requests in the per-individual LWE layout
                 (n = 1024; on average 0.5 TB of outputs each, streamed
                 through the budget in 2,048-output segments), generated
                 inputs, digests."""
    import ctypes as C

    import numpy as np
    import pyoracle
    from idash2019_2_gb300 import gpu
    T = 80882
    w = gpu.synth_model(seed, 16184, T, neighbours=10)
    ctx.set_option("kernel", 4)  # the server runs the warp-specialised kernel (job tables)
    try:
        m = gpu.TrlweModel(ctx, w.model, 3 * 16184, 1024, 1, 1024)
    finally:
        ctx.set_option("kernel", 0)
    rng = np.random.default_rng(seed)

    def draw(k, max_indiv=2000):
        out = []
        for i in range(k):
            length = int(rng.integers(1000, T + 1))
            t0 = int(rng.integers(0, T - length + 1))
            out.append(dict(arrival_s=0.0, n_indiv=int(rng.integers(1, max_indiv + 1)), target_begin=t0,
                            target_end=t0 + length, seed=int(rng.integers(1, 2 ** 62))))
        return out

    # useful multiply-adds of outputs [0, o): prefix sums of per-output terms
    live = (w.model.term_feat != CONSTANT).astype(np.int64)
    term_prefix = np.concatenate([[0], np.cumsum(live)])[w.model.term_ptr.astype(np.int64)]

    def macs(q, row_words, blocks):
        return float(term_prefix[3 * q["target_end"]] - term_prefix[3 * q["target_begin"]]) * row_words * blocks

    def moved(model, q, row_bytes, blocks):
        lo, hi = model.input_rows(3 * q["target_begin"], 3 * q["target_end"])
        return blocks * ((hi - lo) * row_bytes + 3 * (q["target_end"] - q["target_begin"]) * row_bytes)

    def stream(model, qs):
        """Submits qs at their arrival times (seconds after the server
        opened) and waits for all; (results, stats, makespan)."""
        srv = gpu.Server(model, budget, inflight)
        try:
            t_open = time.perf_counter()
            tickets = []
            for q in qs:
                while time.perf_counter() - t_open < q["arrival_s"]:
                    pass
                tickets.append(srv.submit(q["n_indiv"], q["target_begin"], q["target_end"], seed=q["seed"]))
            res = [srv.wait(tk) for tk in tickets]
            st = srv.stats()
        finally:
            srv.close()
        return res, st, max(r["done_s"] for r in res) - qs[0]["arrival_s"]

    def roofline(qs, span, busy_s, row_words, row_bytes, blocks):
        useful = sum(macs(q, row_words(q), blocks(q)) for q in qs)
        alg = sum(moved(m_cur, q, row_bytes(q), blocks(q)) for q in qs)
        roof = compute_roofline(0, useful, 0, alg, span)
        roof["busy_frac"] = busy_s / span
        roof["kernel_imad_frac"] = useful / busy_s / IMAD_PEAK
        roof["kernel_hbm_frac"] = alg / busy_s / 1e9 / peaks()["hbm"]
        return roof, alg

    trlwe_blocks = lambda q: (q["n_indiv"] + 1023) // 1024
    m_cur = m
    calib = draw(64)
    stream(m, calib)
    cres, cst, cspan = stream(m, calib)
    capacity = len(calib) / cspan
    rate = 0.8 * capacity
    reqs = draw(n_requests)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n_requests))
    for r, a in zip(reqs, t):
        r["arrival_s"] = float(a)
    res, st, makespan = stream(m, reqs)
    lat = np.array([r["done_s"] - q["arrival_s"] for r, q in zip(res, reqs)])
    preds = sum(q["n_indiv"] * (q["target_end"] - q["target_begin"]) * 3 for q in reqs)
    roof, req_bytes = roofline(reqs, makespan, st["busy_s"], lambda q: 2048, lambda q: 8192, trlwe_blocks)
    croof, _ = roofline(calib, cspan, cst["busy_s"], lambda q: 2048, lambda q: 8192, trlwe_blocks)
    # CPU: the oracle over the first cpu_requests requests (uniform rows of
    # the same shape; the arithmetic does not depend on the values)
    rows = np.random.default_rng(seed).integers(0, 2 ** 32, size=(3 * 16184, 2048),
                                                dtype=np.uint64).astype(np.uint32).view(np.int32)
    cpu_s, cpu_preds = 0.0, 0
    for q in reqs[:cpu_requests]:
        sub = w.model.slice_outputs(3 * q["target_begin"], 3 * q["target_end"])
        for b in range((q["n_indiv"] + 1023) // 1024):
            ns = min(1024, q["n_indiv"] - 1024 * b)
            t1 = time.perf_counter()
            pyoracle.trlwe_score(sub.term_ptr, sub.term_feat, sub.term_coef, rows, ns, 1, 1024, n_threads=cores())
            cpu_s += time.perf_counter() - t1
            cpu_preds += ns * (q["target_end"] - q["target_begin"]) * 3
    out = {"value": preds / makespan, "requests": n_requests, "requests_per_s": n_requests / makespan,
           "p50_latency_ms": float(np.percentile(lat, 50) * 1e3), "p99_latency_ms": float(np.percentile(lat, 99) * 1e3),
           "arrival_rate_per_s": rate, "capacity_per_s": capacity, "max_inflight": inflight,
           "launches": st["launches"], "roofline": roof,
           "at_capacity": {"requests": len(calib), "value": sum(q["n_indiv"] * (q["target_end"] - q["target_begin"]) * 3
                                                                for q in calib) / cspan,
                           "launches": cst["launches"], "roofline": croof},
           "cpu_baseline": {"value": cpu_preds / cpu_s, "unit": UNIT, "cores": cores(), "kind": "port",
                            "sample": f"{cpu_requests} requests ({cpu_s:.1f} s), oracle restatement"}}

    # end to end: host payloads through page-locked buffers, four requests
    # outstanding from the client's side
    e2e_reqs = draw(e2e_requests)
    slots = 4
    max_in = max(2 * (m.input_rows(3 * q["target_begin"], 3 * q["target_end"])[1] -
                      m.input_rows(3 * q["target_begin"], 3 * q["target_end"])[0]) for q in e2e_reqs) * 8192
    max_out = max(((q["n_indiv"] + 1023) // 1024) * 3 * (q["target_end"] - q["target_begin"]) for q in e2e_reqs) * 8192
    bufs = [(ctx.host_alloc(max_in), ctx.host_alloc(max_out)) for _ in range(slots)]
    for h_in, _ in bufs:
        h_in.array[:] = np.frombuffer(np.random.default_rng(1).bytes(max_in), np.uint8)
    srv = gpu.Server(m, budget, inflight)
    t_open = time.perf_counter()
    inflight_q, lats, h2d, d2h = [], [], 0, 0
    try:
        for i, q in enumerate(e2e_reqs):
            if len(inflight_q) == slots:
                tk, ts = inflight_q.pop(0)
                r = srv.wait(tk)
                lats.append(r["done_s"] - ts)
            h_in, h_out = bufs[i % slots]
            in_shape, out_shape, _ = gpu.serve_input_shape(m, q["n_indiv"], q["target_begin"], q["target_end"])
            n_in, n_out_b = int(np.prod(in_shape)) * 4, int(np.prod(out_shape)) * 4
            a_in = np.ctypeslib.as_array((C.c_uint8 * n_in).from_address(h_in.ptr))
            a_out = np.ctypeslib.as_array((C.c_uint8 * n_out_b).from_address(h_out.ptr))
            ts = time.perf_counter() - t_open
            inflight_q.append((srv.submit(q["n_indiv"], q["target_begin"], q["target_end"], h_in=a_in, h_out=a_out), ts))
            h2d += n_in
            d2h += n_out_b
        for tk, ts in inflight_q:
            r = srv.wait(tk)
            lats.append(r["done_s"] - ts)
        wall = time.perf_counter() - t_open
    finally:
        srv.close()
        for a, b in bufs:
            a.free()
            b.free()
    e2e_preds = sum(q["n_indiv"] * (q["target_end"] - q["target_begin"]) * 3 for q in e2e_reqs)
    out["e2e"] = {"value": e2e_preds / wall, "unit": UNIT, "requests": e2e_requests, "requests_per_s": e2e_requests / wall,
                  "p50_latency_ms": float(np.percentile(lats, 50) * 1e3),
                  "p99_latency_ms": float(np.percentile(lats, 99) * 1e3),
                  "h2d_bytes_per_request": h2d / e2e_requests, "d2h_bytes_per_request": d2h / e2e_requests}
    m.free()

    # the per-individual LWE layout of configuration 5
    ctx.set_option("kernel", 4)
    try:
        lm = gpu.LweModel(ctx, w.model, 3 * 16184, 2000)
    finally:
        ctx.set_option("kernel", 0)
    m_cur = lm
    lreqs = draw(lwe_requests)
    lres, lst, lspan = stream(lm, lreqs)
    llat = [r["done_s"] - q["arrival_s"] for r, q in zip(lres, lreqs)]
    lpreds = sum(q["n_indiv"] * (q["target_end"] - q["target_begin"]) * 3 for q in lreqs)
    lroof, lbytes = roofline(lreqs, lspan, lst["busy_s"], lambda q: q["n_indiv"] * 1025,
                             lambda q: gpu.lwe_row_words(q["n_indiv"]) * 4, lambda q: 1)
    out["lwe"] = {"value": lpreds / lspan, "requests": lwe_requests, "launches": lst["launches"],
                  "p50_latency_ms": float(np.percentile(llat, 50) * 1e3),
                  "p99_latency_ms": float(np.percentile(llat, 99) * 1e3),
                  "bytes_moved": lbytes, "roofline": lroof}
    lm.free()
    return out


def section_decrypt(ctx, model, spec, d_out, seed, steps):
    """Party A's decryption (decrypt_predictions, eval/idash.cpp:682-761) of
    the headline's 242,646 output TRLWE: phase b - a*s at the 1,000 sample
    coefficients, as float, device-resident (CUDA events)."""
    from idash2019_2_gb300 import gpu
    key = gpu.synth_key(seed)
    ns = spec["num_samples"]
    d_dec = ctx.device_alloc(model.n_out * ns * 4)
    run = lambda: gpu.decrypt_device(ctx, key, d_out.ptr, gpu.DENSE_TRLWE, model.n_out, ns, d_dec.ptr)
    for _ in range(3):
        run()
    ms = time_on_stream(ctx, run, steps)
    d_dec.free()
    nz = int(key.sum())
    adds = model.n_out * ns * nz
    return {"value": model.n_out * ns / (ms / 1e3), "unit": "decrypted scores/s", "ms_per_step": ms,
            "key_weight": nz, "word_adds_per_s": adds / (ms / 1e3)}


def section_encrypt(ctx, spec, seed, steps):
    """Party A's encryption (encrypt_data_ph1/ph2, eval/idash.cpp:615-679) of
    the headline's inputs: 16,184 tags x 3 one-hot features = 48,552 fresh
    TRLWE (1,000 genotypes each, 5% missing), device-resident (CUDA events)."""
    import numpy as np
    from idash2019_2_gb300 import gpu
    rng = np.random.default_rng(seed)
    n_tags, ns = spec["n_tags"], spec["num_samples"]
    geno = rng.integers(0, 3, size=(n_tags, ns)).astype(np.int8)
    geno[rng.random(size=geno.shape) < 0.05] = -1
    n_rows = 3 * n_tags
    src = np.arange(n_rows, dtype=np.uint32)  # NUM_REGIONS = 1: row f holds feature f = 3p + v
    d_geno, d_src = ctx.device_alloc(geno.nbytes), ctx.device_alloc(src.nbytes)
    d_geno.upload(geno)
    d_src.upload(src)
    d_out = ctx.device_alloc(n_rows * gpu.RECORD_BYTES)
    key = gpu.synth_key(seed)
    params = gpu.encrypt_params(ns, 1, 1024)
    run = lambda: gpu.encrypt_device(ctx, params, key, seed, n_rows, d_src.ptr, d_geno.ptr, ns, d_out.ptr,
                                     gpu.RECORD_OUT)
    for _ in range(3):
        run()
    ms = time_on_stream(ctx, run, steps)
    for b in (d_geno, d_src, d_out):
        b.free()
    return {"value": n_rows / (ms / 1e3), "unit": "TRLWE encryptions/s", "ms_per_step": ms,
            "key_weight": int(key.sum())}


def section_files(seed, small=False):
    """Rows f1-f4 on files, at the headline's shape (1,000 individuals, 16,184
    tags, 80,882 targets x 3, 5 neighbours):
      - the whole cloud step (idash_cloud_files, eval/cloud.cpp:3-28):
        params.bin, the model directory of one .hr file per output
        (eval/idash.cpp:66-114) and encrypted_data.bin in,
        encrypted_prediction.bin out; three calls: parsing the .hr files, the
        same writing the flattened-model cache, and reading the cache;
      - party A's encryption of the tag genotypes (idash_encrypt_files,
        eval/encrypt.cpp:14-38) and decryption of the predictions to the CSV
        (idash_decrypt_files, eval/decrypt.cpp:13-48).
    Opt-in (about 6 GB of files in the temporary directory)."""
    import shutil
    import tempfile
    from idash2019_2_gb300 import filesets, gpu
    n_indiv, n_tags, n_targets = (1000, 2000, 10000) if small else (1000, 16184, 80882)
    d = tempfile.mkdtemp(prefix="idash_cloud_files_")
    try:
        t0 = time.perf_counter()
        info = filesets.write_cloud_inputs(d, seed, n_indiv, n_tags, n_targets, 5, party_a=True)
        gen_s = time.perf_counter() - t0
        paths = [os.path.join(d, x) for x in ("params.bin", "model", "encrypted_data.bin", "encrypted_prediction.bin")]
        cache = os.path.join(d, "model.cache")
        runs = {}
        for name, use_cache in (("parse_model", False), ("parse_and_write_cache", True), ("model_from_cache", True)):
            if use_cache:
                os.environ["IDASH_MODEL_CACHE"] = cache
            else:
                os.environ.pop("IDASH_MODEL_CACHE", None)
            if os.path.exists(paths[3]):
                os.remove(paths[3])  # each run writes a new prediction file (no truncation of the last)
            t0 = time.perf_counter()
            rep = gpu.cloud_files(*paths)
            wall = time.perf_counter() - t0
            runs[name] = {"wall_s": wall, **{k: rep[k] for k in ("read_s", "plan_s", "score_s", "write_s",
                                                                   "model_from_cache")}}
        os.environ.pop("IDASH_MODEL_CACHE", None)
        out_bytes = os.path.getsize(paths[3])
        in_bytes = os.path.getsize(paths[2])
        keys, csv = os.path.join(d, "keys.bin"), os.path.join(d, "result.csv")
        t0 = time.perf_counter()
        rep = gpu.encrypt_files(keys, os.path.join(d, "tags.txt"), os.path.join(d, "encrypted_data_a.bin"), seed)
        runs["encrypt"] = {"wall_s": time.perf_counter() - t0, **rep}
        t0 = time.perf_counter()
        rep = gpu.decrypt_files(keys, paths[3], csv, False)
        runs["decrypt_to_csv"] = {"wall_s": time.perf_counter() - t0, "csv_bytes": os.path.getsize(csv), **rep}
    finally:
        shutil.rmtree(d, ignore_errors=True)
    preds = info["outputs"] * n_indiv
    best = runs["model_from_cache"]["wall_s"]
    return {"value": preds / best, "unit": UNIT, "s_per_step": best,
            "workload": f"cloud step on files: {n_indiv:,} individuals x {n_targets:,} targets x 3, {n_tags:,} tags, "
                        "5 neighbours (one .hr file per output), wall time of idash_cloud_files",
            "files": {"model_files": info["outputs"], "model_terms": info["terms"], "encrypted_data_bytes": in_bytes,
                      "encrypted_prediction_bytes": out_bytes, "generate_s": gen_s},
            "runs": runs}


def run_sections(ctx, args, sections):
    """The forms beside the headline.  --small shrinks the LWE forms to
    100 individuals x 2,000 tags x 10,000 targets (a few GB on the device),
    the size the ncu captures under profiles/ use."""
    ni, nt, ng = (100, 2000, 10000) if args.small else (1000, 16184, 80882)
    forms = {}
    if "config1" in sections:
        forms["config1"] = section_config1(ctx, args.seed + 5)
    # serving before the LWE and integer-polynomial forms: its host-payload
    # leg pins about 20 GB of host memory, and after those forms' 100+ GB
    # device working sets its copies measured at half the host link's rate
    if "serving" in sections:
        forms["serving"] = section_serving(ctx, args.seed + 2, **(
            dict(n_requests=300, e2e_requests=20, lwe_requests=2, cpu_requests=2) if args.small else {}))
    if "lwe_full" in sections:
        forms["lwe_full"] = section_lwe(ctx, args.seed, ni, nt, ng, neighbours=5, cpu_outputs=512)
    if "batched_uneven" in sections:
        forms["batched_uneven"] = section_lwe(ctx, args.seed + 1, ni, nt, ng, choices=[5, 10, 20, 30, 50], passes=1,
                                              cpu_outputs=192)
    if "intpoly" in sections:
        forms["intpoly"] = section_intpoly(ctx, args.seed + 3, scale=64 if args.small else 1)
    if "files" in sections:
        forms["files"] = section_files(args.seed + 4, small=args.small)
    return forms


FORM_WORKLOADS = {
    "plain": "the headline workload through the plain per-output kernel (k_score_direct)",
    "kinds": "the headline workload through each batched kernel kind, ms per pass",
    "config1": "100 individuals x 2,000 targets x 3, 500 tags, 5 neighbours: TRLWE-packed (NUM_REGIONS 10, "
               "REGION_SIZE 102) and per-individual LWE (n=1024, 0.62 GB in, 2.46 GB out)",
    "lwe_full": "per-individual LWE at full scale: 1,000 individuals x 80,882 targets x 3, 16,184 tags, 5 neighbours, "
                "n=1024 (199 GB in, 995 GB out per pass, outputs through a 2-buffer HBM ring)",
    "batched_uneven": "per-individual LWE at full scale, neighbours uniform from {5,10,20,30,50}",
    "intpoly": "integer-polynomial x TRLWE: 48,552 input TRLWE, 242,646 outputs, 60 dense int16 weight polynomials "
               "per output, N=1024, predictions = outputs x 1,024",
    "serving": "online server, 10 neighbours, 150 GB HBM budget, individuals ~ U[1,2000], targets ~ U[1000, 80882] "
               "contiguous: 10,000 Poisson requests at 0.8 x capacity (TRLWE-packed, device-generated inputs, "
               "digests); e2e: 200 requests with host payloads in page-locked memory; lwe: 12 requests in the "
               "per-individual LWE layout (n=1024), generated inputs, digests",
    "encrypt": "party A encryption of the headline's 48,552 input TRLWE",
    "decrypt": "party A decryption of the headline's 242,646 outputs x 1,000 scores",
}


def run_sections_only(args):
    """--no-headline: only the listed sections, one JSON line of forms."""
    import torch
    from idash2019_2_gb300 import gpu
    torch.cuda.init()
    ctx = gpu.Context(0)
    sections = set(args.sections.split(",")) if args.sections else set()
    forms = run_sections(ctx, args, sections)
    ctx.close()
    print(json.dumps(sig({"metric": METRIC, "unit": UNIT, "forms": forms})), flush=True)


def run_ours(args):
    import numpy as np
    import torch
    from idash2019_2_gb300 import gpu
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.init()
    spec = workload_spec(args.workload)
    ctx = gpu.Context(local)
    w = gpu.synth_model(args.seed + rank, spec["n_tags"], spec["n_targets"], neighbours=spec["neighbours"])
    params = gpu.TrlweParams(1024, 1, spec["num_samples"], spec["regions"], spec["region_size"], 1 << 18, 42)
    if args.kernel is not None:
        ctx.set_option("kernel", args.kernel)
    model = gpu.TrlweModel(ctx, w.model, spec["n_rows"], spec["num_samples"], spec["regions"], spec["region_size"])
    d_in = ctx.device_alloc(spec["n_rows"] * 8192)
    d_out = ctx.device_alloc(model.n_out * 8192)
    gpu.synth_trlwe_device(ctx, args.seed + rank, params, spec["n_tags"], d_in.ptr, gpu.DENSE_TRLWE)
    ctx.sync()
    lay = gpu.DENSE_TRLWE
    for _ in range(max(args.warmup, 3)):
        model.score_device(d_in.ptr, lay, d_out.ptr, lay)
    ctx.sync()
    info = model.info()

    stream = torch.cuda.ExternalStream(ctx.stream)
    sampler = ClockSampler(local)
    time.sleep(0.3)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    ctx.sync()
    launches0 = ctx.stats()["kernel_launches"]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.time()
    e0.record(stream)
    with timed_range():
        for _ in range(args.steps):
            model.score_device(d_in.ptr, lay, d_out.ptr, lay)
    e1.record(stream)
    e1.synchronize()
    t1 = time.time()
    ctx.sync()
    torch.cuda.synchronize()
    launches = ctx.stats()["kernel_launches"] - launches0
    ms = max_over_ranks(e0.elapsed_time(e1))
    time.sleep(0.25)
    clocks = sampler.summary(t0, t1)
    sampler.stop()
    preds_per_step = spec["n_indiv"] * spec["n_targets"] * 3
    ms_step = ms / args.steps
    value = preds_per_step * world / (ms_step / 1e3)

    alg_bytes = trlwe_alg_bytes(info, model.n_out)
    roof = hbm_roofline(alg_bytes, ms_step / 1e3)
    # DRAM bytes of one launch of the kernel kind the autotuner chose, from its
    # ncu capture on this workload (null when that kind has none)
    roof["traffic"] = profiled_traffic({0: "trlwe_window_full.txt", 2: "trlwe_pipe_full.txt",
                                        3: "trlwe_ws_full.txt"}.get(info["kernel"], ""))
    roof["algorithmic_bytes_per_launch"] = alg_bytes
    useful = float(np.count_nonzero(w.model.term_feat != CONSTANT)) * 2048
    roof["imad_frac"] = useful / (ms_step / 1e3) / IMAD_PEAK

    # end to end through the host-memory entry point
    e2e_steps = max(3, min(args.steps, 20))
    h_in = ctx.host_alloc(spec["n_rows"] * 8192)
    h_out = ctx.host_alloc(model.n_out * 8192)
    h_in.array[:] = d_in.download()
    model.score_host(h_in.ptr, lay, spec["n_rows"], h_out.ptr, lay)
    st0 = ctx.stats()
    if world > 1:
        torch.distributed.barrier()
    te0 = time.perf_counter()
    for _ in range(e2e_steps):
        model.score_host(h_in.ptr, lay, spec["n_rows"], h_out.ptr, lay)
    te = max_over_ranks(time.perf_counter() - te0)
    st1 = ctx.stats()
    e2e = {"value": preds_per_step * world * e2e_steps / te, "unit": UNIT,
           "h2d_bytes_per_step": (st1["h2d_bytes"] - st0["h2d_bytes"]) // e2e_steps,
           "d2h_bytes_per_step": (st1["d2h_bytes"] - st0["d2h_bytes"]) // e2e_steps,
           "ms_per_step": te / e2e_steps * 1e3}

    base = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rows = np.frombuffer(h_in.array, dtype=np.int32).reshape(spec["n_rows"], 2048)
        base = cpu_trlwe(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, spec, 8.0)
    h_in.free()
    h_out.free()

    forms = {}
    sections = set(args.sections.split(",")) if args.sections else set()
    if world == 1 and "plain" in sections:
        forms["plain"] = section_plain(ctx, w, spec, d_in, d_out, min(args.steps, 200))
        forms["plain"]["batched_over_plain"] = value / forms["plain"]["value"]
    if world == 1 and "kinds" in sections:
        forms["kinds"] = section_kinds(ctx, w, spec, d_in, d_out, min(args.steps, 200))
    if world == 1 and "decrypt" in sections:
        forms["decrypt"] = section_decrypt(ctx, model, spec, d_out, args.seed + rank, min(args.steps, 50))
    if world == 1 and "encrypt" in sections:
        forms["encrypt"] = section_encrypt(ctx, spec, args.seed + rank, min(args.steps, 50))
    d_in.free()
    d_out.free()
    model.free()
    if world == 1:
        forms.update(run_sections(ctx, args, sections - {"plain", "kinds", "decrypt", "encrypt"}))

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": value / PUBLISHED_PREDICTIONS_PER_S if args.workload == "trlwe_full" else None,
                "dtype": "int32 (Z/2^32)", "data": "synthetic (seeded)", "config": config_of(spec, world),
                "kernel": {"name": KERNEL_NAMES.get(info["kernel"], str(info["kernel"])),
                           "slice_words": info["slice_words"]},
                "roofline": roof, "cpu_baseline": base, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
        if forms:
            line["forms"] = forms
            line["form_workloads"] = {k: FORM_WORKLOADS[k] for k in forms if k in FORM_WORKLOADS}
        print(json.dumps(sig(line)), flush=True)
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="trlwe_full")
    ap.add_argument("--seed", type=int, default=0x1DA52019)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sections",
                    default="plain,kinds,config1,encrypt,decrypt,lwe_full,batched_uneven,intpoly,serving",
                    help="extra forms measured after the headline (comma list, '' for none; 'files', the "
                         "cloud step through its files, is opt-in)")
    ap.add_argument("--no-headline", action="store_true",
                    help="measure only --sections (no headline, e2e or CPU baseline)")
    ap.add_argument("--small", action="store_true",
                    help="LWE and int-poly sections at a reduced size, serving with fewer requests (profiling)")
    ap.add_argument("--kernel", type=int, default=None,
                    help="the headline model's kernel option (idash_set_option 'kernel'; default: autotuned)")
    args = ap.parse_args()
    args.steps_given = args.steps is not None
    if args.steps is None:
        args.steps = 2000
    if args.impl == "reference":
        run_reference(args)
    elif args.no_headline:
        run_sections_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

#!/usr/bin/env python3
"""Encrypted predictions/s of the party-B scoring step (cloud_compute_score,
eval/idash.cpp:763-848) on GB300.

One step = one pass of the scoring step over one batch: every output
ciphertext of the model computed once.  Default workload (full scale, the
reference's TRLWE-packed layout): 1,000 individuals packed in one region per
TRLWE (N = 1024), 16,184 tag SNPs (48,552 input TRLWE), 80,882 targets x 3
outputs (242,646 output TRLWE), 5 nearest-tag neighbours, coefficients
uniform in [-8192, 8191]; synthetic seeded data.

  value   predictions/s with inputs and model resident in HBM (CUDA events
          on the launching stream; inputs 0.4 GB > L2, outputs 2 GB)
  e2e     the same through idash_score_trlwe_host with page-locked host
          buffers: every step copies the inputs in and the outputs out
  roofline the scoring kernel against the measured HBM copy bandwidth
  cpu_baseline the oracle's restatement of the reference loop on the host cores

--impl reference times that CPU restatement alone (all host threads) on the
same workload and prints the same line with impl=reference.
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
KERNEL_NAMES = {0: "window (batched, persistent, CUDA graph)", 1: "direct (plain)",
                2: "pipe (batched, double-buffered, persistent, CUDA graph)",
                3: "ws (batched, warp-specialised producer + consumers over an mbarrier ring, CUDA graph)",
                4: "tc (batched, tensor cores: exact fp16 digit products on tcgen05.mma, fp32 accumulators in TMEM, "
                   "CUDA graph)"}


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
    try:
        p = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


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


def cpu_baseline(model_csr, rows, spec, min_seconds=10.0, max_reps=1000):
    """The oracle's restatement of the reference loop (OpenMP over outputs,
    eval/idash.cpp:779-842) on all host cores, full workload per rep."""
    import pyoracle
    cores = os.cpu_count() or 1
    preds = spec["n_indiv"] * spec["n_targets"] * 3
    reps, t0 = 0, time.perf_counter()
    while True:
        pyoracle.trlwe_score(model_csr.term_ptr, model_csr.term_feat, model_csr.term_coef, rows, spec["num_samples"],
                             spec["regions"], spec["region_size"], n_threads=cores)
        reps += 1
        el = time.perf_counter() - t0
        if el >= min_seconds or reps >= max_reps:
            break
    return {"value": preds * reps / el, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{reps} full passes of the workload ({el:.1f} s), oracle/oracle.c restatement of "
                      f"eval/idash.cpp:779-842, OpenMP {cores} threads"}


def workload_spec(name):
    spec = dict(WORKLOADS[name])
    regions = max(1, 1024 // spec["n_indiv"])
    spec.update(regions=regions, region_size=1024 // regions, num_samples=spec["n_indiv"],
                n_rows=(3 * spec["n_tags"] + regions - 1) // regions)
    return spec


def run_reference(args):
    import numpy as np
    from idash2019_2_gb300 import gpu
    rank, world, _ = dist_env()
    if rank != 0:
        return
    spec = workload_spec(args.workload)
    w = gpu.synth_model(args.seed, spec["n_tags"], spec["n_targets"], neighbours=spec["neighbours"])
    rng = np.random.default_rng(args.seed)
    rows = rng.integers(0, 2 ** 32, size=(spec["n_rows"], 2048), dtype=np.uint64).astype(np.uint32).view(np.int32)
    import pyoracle
    preds = spec["n_indiv"] * spec["n_targets"] * 3
    cores = os.cpu_count() or 1
    for _ in range(args.warmup):
        pyoracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, spec["num_samples"],
                             spec["regions"], spec["region_size"], n_threads=cores)
    steps = args.steps if args.steps_given else 3
    t0 = time.perf_counter()
    for _ in range(steps):
        pyoracle.trlwe_score(w.model.term_ptr, w.model.term_feat, w.model.term_coef, rows, spec["num_samples"],
                             spec["regions"], spec["region_size"], n_threads=cores)
    el = time.perf_counter() - t0
    value = preds * steps / el
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": steps, "warmup": args.warmup,
            "ms_per_step": el / steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": value / PUBLISHED_PREDICTIONS_PER_S if args.workload == "trlwe_full" else None,
            "dtype": "int32 (Z/2^32)", "data": "synthetic (seeded)", "impl": "reference",
            "config": {"workload": spec["desc"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{steps} full passes; oracle/oracle.c restatement of eval/idash.cpp:779-842 "
                                       f"(the reference's TFHE dependency is absent, so its cloud binary cannot be "
                                       f"built on this host)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
        m.free()
    finally:
        ctx.set_option("kernel", 0)
    preds = spec["n_indiv"] * spec["n_targets"] * 3
    return {"value": preds / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
            "kernel": "direct: one output per team, every input read from global memory"}


def section_kinds(ctx, w, spec, d_in, d_out, steps):
    """Each batched kernel kind on the headline workload, autotuned within its
    kind (slice width, CTAs per SM, ring depth)."""
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
            ms = time_on_stream(ctx, lambda: m.score_device(d_in.ptr, lay, d_out.ptr, lay), steps)
            info = m.info()
            out[name] = {"ms_per_step": ms, "slice_words": info["slice_words"], "n_blocks": info["n_blocks"],
                         "max_window_slots": info["max_window_slots"]}
            m.free()
        finally:
            ctx.set_option("kernel", 0)
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
            "rows": model.n_out, "samples": ns, "key_weight": nz,
            "word_adds_per_s": adds / (ms / 1e3),
            "kernel": "k_decrypt_binary: 4 rows per CTA, negacyclic extension of each mask in (bank-padded) "
                      "shared memory, 16 consecutive coefficients per thread, the key in 32-position chunks: a "
                      "48-word window in registers per chunk, one uniform branch per key bit"}


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
    return {"value": n_rows / (ms / 1e3), "unit": "TRLWE encryptions/s", "ms_per_step": ms, "rows": n_rows,
            "samples": ns, "key_weight": int(key.sum()),
            "kernel": "k_encrypt_binary: 4 rows per CTA, counter-based mask and Box-Muller noise, mask*key as a "
                      "register-windowed product (16 coefficients per thread), one-hot messages, record headers"}


def section_lwe(ctx, name, seed, n_indiv, n_tags, n_targets, neighbours=5, choices=None, passes=2, chunk=2048):
    """Per-individual LWE form: inputs resident (n_indiv LWE samples of n=1024
    per feature row), outputs produced range by range into a 2-slot HBM ring
    (the full output does not fit in HBM)."""
    from idash2019_2_gb300 import gpu
    w = gpu.synth_model(seed, n_tags, n_targets, neighbours=neighbours, choices=choices)
    n_feat = 3 * n_tags
    stride = gpu.lwe_row_words(n_indiv)
    L = n_indiv * 1025
    d_in = ctx.device_alloc(n_feat * stride * 4)
    gpu.synth_lwe_device(ctx, seed, 1024, n_indiv, n_feat, d_in.ptr, stride)
    m = gpu.LweModel(ctx, w.model, n_feat, n_indiv)
    ring = [ctx.device_alloc(chunk * stride * 4) for _ in range(2)]
    ranges = [(lo, min(lo + chunk, m.n_out)) for lo in range(0, m.n_out, chunk)]

    def one_pass():
        for c, (lo, hi) in enumerate(ranges):
            m.score_device(n_indiv, d_in.ptr, stride, lo, hi, ring[c % 2].ptr, stride)

    t0 = time.perf_counter()
    one_pass()  # first call autotunes the slice width
    ctx.sync()
    first_s = time.perf_counter() - t0
    launches0 = ctx.stats()["kernel_launches"]
    ms = time_on_stream(ctx, one_pass, passes)
    launches = (ctx.stats()["kernel_launches"] - launches0) // passes
    info = m.info()
    preds = n_indiv * n_targets * 3
    alg = info["algorithmic_in_rows"] * L * 4 + m.n_out * L * 4 + info["n_terms"] * 8 + m.n_out * 8
    peak, _ = peaks()
    macs = float(sum(int(w.model.term_ptr[o + 1] - w.model.term_ptr[o]) - 1 for o in range(0, m.n_out, 97))) * 97
    out = {"value": preds / (ms / 1e3), "unit": UNIT, "ms_per_step": ms, "workload": name,
           "individuals": n_indiv, "targets": n_targets, "tags": n_tags,
           "neighbours": neighbours if not choices else f"uniform from {choices}",
           "input_bytes": n_feat * stride * 4, "output_bytes_per_step": m.n_out * L * 4,
           "kernel": KERNEL_NAMES.get(info["kernel"], str(info["kernel"])),
           "slice_words": info["slice_words"], "launches_per_step": launches,
           "first_pass_s_including_autotune": first_s,
           "roofline": {"bound": "hbm", "achieved": alg / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": alg / (ms / 1e3) / 1e9 / peak, "algorithmic_bytes_per_step": alg},
           "int_macs_per_step_est": macs * L, "imad_tops_at_this_rate": macs * L / (ms / 1e3) / 1e12}
    for b in ring:
        b.free()
    d_in.free()
    m.free()
    return out


def section_intpoly(ctx, seed, passes=5, scale=1):
    """Integer-polynomial x TRLWE product at full scale: 48,552 input TRLWE
    (16,184 tags x 3), 242,646 outputs (80,882 targets x 3), 20 neighbours
    (60 dense int16 weight polynomials per output, |w| <= 8192), one block of
    1,024 individuals per TRLWE.  Exact (two-prime NTT + CRT).  scale > 1
    divides the tag and target counts (profiling size)."""
    import numpy as np
    from idash2019_2_gb300 import gpu
    n_tags, n_targets = 16184 // scale, 80882 // scale
    w = gpu.synth_model(seed, n_tags, n_targets, neighbours=20)
    csr = w.model
    const = csr.term_feat == 0xFFFFFFFF
    counts = np.diff(csr.term_ptr.astype(np.int64)) - np.add.reduceat(const.astype(np.int64),
                                                                        csr.term_ptr[:-1].astype(np.int64))
    ptr = np.concatenate([[0], np.cumsum(counts)]).astype(np.uint64)
    feat = csr.term_feat[~const]
    bias = np.zeros(csr.n_out, np.int32)
    owner = np.repeat(np.arange(csr.n_out), np.diff(csr.term_ptr.astype(np.int64)))
    bias[owner[const]] = csr.term_coef[const]
    icsr = gpu.CSRModel(ptr, feat, np.zeros(len(feat), np.int32))
    n_terms, n_rows = len(feat), 3 * n_tags
    d_poly = ctx.device_alloc(n_terms * 1024 * 2)
    gpu.synth_int16_device(ctx, seed, n_terms * 1024, 8192, d_poly.ptr)
    t0 = time.perf_counter()
    m = gpu.IntpolyModel(ctx, icsr, d_poly.ptr, n_rows, 1024, 1024, bias=bias, poly_on_device=True)
    build_s = time.perf_counter() - t0
    d_poly.free()
    params = gpu.TrlweParams(1024, 1, 1024, 1, 1024, 1 << 18, 42)
    d_in = ctx.device_alloc(n_rows * 8192)
    gpu.synth_trlwe_device(ctx, seed, params, n_tags, d_in.ptr, gpu.DENSE_TRLWE)
    d_out = ctx.device_alloc(csr.n_out * 8192)
    run = lambda: m.score_device(d_in.ptr, gpu.DENSE_TRLWE, 0, csr.n_out, d_out.ptr, gpu.DENSE_TRLWE)
    run()
    ms = time_on_stream(ctx, run, passes)
    # compulsory traffic of this algorithm per pass: the NTT-domain weights
    # (2 primes x N words per term), input rows in and their NTT out and back
    # in, output rows out
    traffic = n_terms * 2 * 1024 * 4 + n_rows * 8192 + 2 * n_rows * 4 * 1024 * 4 + csr.n_out * 8192
    peak, _ = peaks()
    out = {"value": csr.n_out * 1024 / (ms / 1e3), "unit": UNIT, "ms_per_step": ms,
           "outputs_per_s": csr.n_out / (ms / 1e3), "terms": n_terms, "model_build_s": build_s,
           "schoolbook_mac_per_s": n_terms * 2 * 1024 * 1024 / (ms / 1e3),
           "resident_weight_bytes": n_terms * 2 * 1024 * 4,
           "roofline": {"bound": "hbm", "achieved": traffic / (ms / 1e3) / 1e9, "peak": peak, "unit": "GB/s",
                        "frac": traffic / (ms / 1e3) / 1e9 / peak, "algorithmic_bytes_per_step": traffic},
           "workload": f"integer-polynomial x TRLWE: {n_rows:,} input TRLWE, {csr.n_out:,} outputs, 60 dense int16 "
                       "weight polynomials per output, N=1024, 1,024 individuals per TRLWE (predictions = outputs x "
                       "1024)"}
    for b in (d_in, d_out):
        b.free()
    m.free()
    return out


def section_serving(ctx, seed, n_requests=10000, budget=150 << 30, inflight=4):
    """Continuous batching (idash_serve_trlwe) over a Poisson stream: each
    request has individuals ~ U[1, 2000] and a contiguous target range of
    length ~ U[1000, 80882]; 10 neighbours; model and index tables resident;
    150 GB HBM admission budget.  The arrival rate is 0.8 x the measured
    capacity (64 requests arriving at once)."""
    import numpy as np
    from idash2019_2_gb300 import gpu
    T = 80882
    w = gpu.synth_model(seed, 16184, T, neighbours=10)
    m = gpu.TrlweModel(ctx, w.model, 3 * 16184, 1024, 1, 1024)
    rng = np.random.default_rng(seed)

    def draw(k):
        out = []
        for i in range(k):
            length = int(rng.integers(1000, T + 1))
            t0 = int(rng.integers(0, T - length + 1))
            out.append(dict(arrival_s=0.0, n_indiv=int(rng.integers(1, 2001)), target_begin=t0,
                            target_end=t0 + length, seed=int(rng.integers(1, 2 ** 62))))
        return out

    calib = draw(64)
    res, _ = m.serve(calib, budget, inflight)  # includes the one-off autotune
    res, _ = m.serve(calib, budget, inflight)
    capacity = len(calib) / max(r["done_s"] for r in res)
    rate = 0.8 * capacity
    reqs = draw(n_requests)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n_requests))
    for r, a in zip(reqs, t):
        r["arrival_s"] = float(a)
    t0 = time.perf_counter()
    res, _ = m.serve(reqs, budget, inflight)
    wall = time.perf_counter() - t0
    lat = np.array([r["done_s"] - q["arrival_s"] for r, q in zip(res, reqs)])
    makespan = max(r["done_s"] for r in res) - reqs[0]["arrival_s"]
    preds = sum(q["n_indiv"] * (q["target_end"] - q["target_begin"]) * 3 for q in reqs)
    m.free()
    return {"value": preds / makespan, "unit": UNIT, "requests": n_requests, "requests_per_s": n_requests / makespan,
            "p50_latency_ms": float(np.percentile(lat, 50) * 1e3), "p99_latency_ms": float(np.percentile(lat, 99) * 1e3),
            "mean_latency_ms": float(lat.mean() * 1e3), "arrival_rate_per_s": rate,
            "capacity_per_s": capacity, "hbm_budget_bytes": budget, "max_inflight": inflight,
            "mean_request_device_bytes": float(np.mean([r["device_bytes"] for r in res])),
            "wall_s": wall,
            "workload": "Poisson stream of 10,000 requests: individuals ~ U[1,2000] (TRLWE-packed, 1,024 per "
                        "block), contiguous targets of length ~ U[1000, 80882], 10 neighbours, 150 GB HBM budget; "
                        "request ciphertexts generated on the device"}


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
    scale = f"{ni:,} individuals x {ng:,} targets x 3, {nt:,} tags"
    forms = {}
    if "lwe_full" in sections:
        forms["lwe_full"] = section_lwe(ctx, f"per-individual LWE: {scale}, 5 neighbours, n=1024", args.seed,
                                        ni, nt, ng, neighbours=5)
    if "batched_uneven" in sections:
        forms["batched_uneven"] = section_lwe(ctx, f"batched uneven neighbourhoods, per-individual LWE: {scale}, "
                                                   "neighbours uniform from {5,10,20,30,50}", args.seed + 1,
                                              ni, nt, ng, choices=[5, 10, 20, 30, 50], passes=1)
    if "intpoly" in sections:
        forms["intpoly"] = section_intpoly(ctx, args.seed + 3, scale=64 if args.small else 1)
    if "serving" in sections:
        forms["serving"] = section_serving(ctx, args.seed + 2)
    if "files" in sections:
        forms["files"] = section_files(args.seed + 4, small=args.small)
    return forms


def run_sections_only(args):
    """--no-headline: only the listed sections, one JSON line of forms."""
    import torch
    from idash2019_2_gb300 import gpu
    torch.cuda.init()
    ctx = gpu.Context(0)
    sections = set(args.sections.split(",")) if args.sections else set()
    forms = run_sections(ctx, args, sections)
    ctx.close()
    print(json.dumps({"metric": METRIC, "unit": UNIT, "forms": forms}), flush=True)


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

    # algorithmic bytes of one launch: each distinct input TRLWE read once,
    # each output TRLWE written once, the model's CSR (4 B feature + 4 B
    # coefficient per term, 4 B bias + 4 B row pointer per output)
    alg_bytes = info["algorithmic_in_rows"] * 8192 + model.n_out * 8192 + info["n_terms"] * 8 + model.n_out * 8
    peak, peak_src = peaks()
    achieved = alg_bytes / (ms_step / 1e3) / 1e9
    # DRAM bytes of one launch of the kernel kind the autotuner chose, from its
    # ncu capture on this workload (null when that kind has none)
    traffic = profiled_traffic({0: "trlwe_window_full.txt", 2: "trlwe_pipe_full.txt",
                                3: "trlwe_ws_full.txt"}.get(info["kernel"], ""))

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
        base = cpu_baseline(w.model, rows, spec)
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
                "dtype": "int32 (Z/2^32)", "data": "synthetic (seeded)",
                "config": {"workload": spec["desc"], "individuals": spec["n_indiv"], "targets": spec["n_targets"],
                           "tags": spec["n_tags"], "neighbours": spec["neighbours"], "outputs": model.n_out,
                           "input_rows": spec["n_rows"], "l2": "inputs 0.40 GB and outputs 1.99 GB exceed the 129 MB L2",
                           "kernel": KERNEL_NAMES.get(info["kernel"], str(info["kernel"])),
                           "slice_words": info["slice_words"], "parallelism": f"{world} independent batch(es)"},
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_source": peak_src,
                             "algorithmic_bytes_per_launch": alg_bytes},
                "cpu_baseline": base, "e2e": e2e, "gpu_launches": launches, "clocks": clocks}
        if forms:
            line["forms"] = forms
        print(json.dumps(line), flush=True)
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
    ap.add_argument("--sections", default="plain,kinds,encrypt,decrypt,lwe_full,batched_uneven,intpoly,serving",
                    help="extra forms measured after the headline (comma list, '' for none; 'files', the "
                         "cloud step through its files, is opt-in)")
    ap.add_argument("--no-headline", action="store_true",
                    help="measure only --sections (no headline, e2e or CPU baseline)")
    ap.add_argument("--small", action="store_true", help="LWE sections at a reduced size (profiling)")
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

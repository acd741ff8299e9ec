#!/usr/bin/env python
"""Benchmark of the FX correlator hot path on one GB300 (or N replicas).

Workload (default): c2_station40 -- NE=40 inputs, Nch=2048, Ntaps=8,
Nspectra=4096, 16 integrations streamed back to back with the PFB history
carried between them; synthetic int8 I/Q from the integer generator.
One step = the 16 integrations (fused F-engine + Hermitian X-engine per
integration, through the plan API).  Metric: antenna-samples/s =
NE * Nspectra * Nch * 16 / step time.  The 10.7 GB input stream is larger
than L2, so no L2 flush is needed between steps.

  value      device-timed (CUDA events on the plan's stream), inputs resident
  e2e        same metric through mdt_fx_execute_host: pinned host samples in,
             host visibilities out, copies inside the timed region
  roofline   the dominant kernel, achieved from live CUDA-event kernel times
  cpu_baseline  the oracle's FP32 OpenMP pipeline on a bounded sample (rank 0)

--impl reference times the reference path's CPU implementation on the host
cores.  The reference has no CPU FX code, so this is the oracle port (FP32,
OpenMP, all host threads) on a bounded sample of the same workload.

Multi-GPU (torchrun): replicas only -- rank r runs integrations
[16r, 16r + 16) of one stream (its own span of the counter-based generator,
lead-in included), no data-path collective; value = all ranks' samples / max
rank time ("scaling": "weak").
"""
import argparse
import importlib
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# DRAM bytes (read + write) per launch of the FP32 path's kernels on the c2
# workload, from ncu captures of one c2 integration (profiles/fengine_c64b_c2.txt,
# profiles/xengine_herm_f32_c2.txt); the per-launch work of the bench is the
# same integration, so no scaling is needed.
NCU_TRAFFIC = {"fengine_c64b": 677.995e6 + 2637.297e6,
               "xengine_herm_f32": 2684.435e6 + 26.480e6}
# The tensor path's kernels on one c3 integration (Nsp = 8192), scaled from ncu
# captures at Nsp = 1024 (profiles/fengine_tc_c3.txt, profiles/xengine_tc_c3.txt):
# the F-engine's reads and writes and the X-engine's operand reads grow with
# the spectra processed, the X-engine's visibility writes do not.
NCU_TRAFFIC_C3 = {"fengine_tc": 0.555248e9 * 8199 / 1031 + 1.022932e9 * 8,
                  "xengine_tc": 1.076980e9 * 8 + 0.484042e9}


def bind_to_gpu_cpus(gpu_index):
    """Restricts this process to the CPUs local to the GPU (sysfs local_cpulist
    of its PCI device), so that pinned host buffers are allocated on the
    GPU's NUMA node.  Returns the CPU list text, or None when unavailable."""
    try:
        bus = subprocess.run(["nvidia-smi", "-i", str(gpu_index), "--query-gpu=pci.bus_id",
                              "--format=csv,noheader"], capture_output=True, text=True,
                             timeout=30).stdout.strip().lower()
        if not bus:
            return None
        dom, rest = bus.split(":", 1)
        path = "/sys/bus/pci/devices/%s:%s/local_cpulist" % (dom[-4:], rest)
        text = open(path).read().strip()
        cpus = set()
        for part in text.split(","):
            lo, _, hi = part.partition("-")
            cpus.update(range(int(lo), int(hi or lo) + 1))
        if cpus:
            os.sched_setaffinity(0, cpus)
            return text
    except (OSError, ValueError, subprocess.SubprocessError):
        return None
    return None


def load_pkg():
    return importlib.import_module("mdt_fpga-gpu_pipeline_gb300")


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), d.get("bf16_tflops", 1900.0), "measured"
    return 6800.0, 1900.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.proc = None
        self.path = os.path.join("/tmp", "mdt_clocks_%d_%d.csv" % (os.getpid(), gpu_index))

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    smax.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def cpu_pipeline_rate(cfg, budget_s, threads=None):
    """Oracle FP32 OpenMP pipeline on the host: (samples/s, sample text, cores)."""
    from oracle import oracle
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    ne, nch, ntaps = cfg.nelements, cfg.nchannels, cfg.ntaps
    cores = int(os.environ.get("OMP_NUM_THREADS", os.cpu_count() or 1))
    win = oracle.window_hamming_sinc(nch, ntaps)

    def run(nsp):
        iq = oracle.synth_iq(cfg.seed, ne, nch, 0, nsp + ntaps - 1, cfg.sigma_q8(),
                             cfg.tone_q16())
        t0 = time.perf_counter()
        oracle.fx(iq, win, ne, nch, ntaps, nsp, double=False)
        return time.perf_counter() - t0

    probe = 32
    dt = run(probe)
    nsp = int(max(64, min(cfg.nspectra, probe * budget_s / max(dt, 1e-3))))
    dt = run(nsp)
    rate = ne * nsp * nch / dt
    sample = ("%s shape (NE=%d, Nch=%d, Ntaps=%d), first %d of %d spectra of one integration, "
              "all channels, FP32 OpenMP oracle pipeline" % (cfg.name, ne, nch, ntaps, nsp,
                                                              cfg.nspectra))
    return rate, sample, cores, nsp


def run_reference(args, cfg):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    ne, nch, ntaps = cfg.nelements, cfg.nchannels, cfg.ntaps
    cores = os.cpu_count() or 1
    win = oracle.window_hamming_sinc(nch, ntaps)
    # size each step to ~3 s of CPU work
    iq = oracle.synth_iq(cfg.seed, ne, nch, 0, 32 + ntaps - 1, cfg.sigma_q8(), cfg.tone_q16())
    t0 = time.perf_counter()
    oracle.fx(iq, win, ne, nch, ntaps, 32, double=False)
    per_sp = (time.perf_counter() - t0) / 32
    nsp = int(max(32, min(cfg.nspectra, 3.0 / max(per_sp, 1e-6))))
    iq = oracle.synth_iq(cfg.seed, ne, nch, 0, nsp + ntaps - 1, cfg.sigma_q8(), cfg.tone_q16())
    for _ in range(args.warmup):
        oracle.fx(iq, win, ne, nch, ntaps, nsp, double=False)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        oracle.fx(iq, win, ne, nch, ntaps, nsp, double=False)
    dt = (time.perf_counter() - t0) / args.steps
    value = ne * nsp * nch / dt
    sample = ("%s shape, %d of %d spectra of one integration per step, all channels" %
              (cfg.name, nsp, cfg.nspectra))
    line = {
        "impl": "reference", "metric": "F+X engine antenna-samples/s", "value": value,
        "unit": "antenna-samples/s", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": cfg.name, "nelements": ne, "nchannels": nch, "ntaps": ntaps,
                   "nspectra": cfg.nspectra, "integrations": cfg.nint,
                   "sample_spectra_per_step": nsp},
        "cpu_baseline": {"value": value, "unit": "antenna-samples/s", "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": "antenna-samples/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": "the reference has no CPU FX implementation; this is the oracle's FP32 "
                "OpenMP restatement of its GPU sequence on all host threads",
    }
    print(json.dumps(line))


def measure_plan(mdt, cfg, precision, dev, steps, warmup, seed_offset=0):
    """Device-timed streamed FX over cfg.nint integrations with the plan API.
    Returns (ms per step, F-engine ms per launch, X-engine ms per launch,
    plan scale)."""
    import torch
    ne, nch, ntaps, nsp, nint = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra, cfg.nint
    sb = ne * nch * 2
    total_sp = nint * nsp + ntaps - 1

    def t(a):
        return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    iq = torch.empty(total_sp * sb, dtype=torch.int8, device=dev)
    ssig, sdel = cfg.sources()
    mdt.synth_iq(cfg.seed + seed_offset, ne, nch, 0, total_sp, t(cfg.sigma_q8()), iq,
                 tone_q16=t(cfg.tone_q16()), src_sigma_q8=t(ssig), src_delay=t(sdel))
    win = torch.empty(nch * ntaps, dtype=torch.float32, device=dev)
    mdt.window_hamming_sinc(nch, ntaps, win)
    vis = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=precision, stream=stream)
    plan.set_window(win)
    first = (nsp + ntaps - 1) * sb

    def step():
        plan.stream_reset()
        plan.stream_push(iq[:first], vis[0])
        for j in range(1, nint):
            lo = (j * nsp + ntaps - 1) * sb
            plan.stream_push(iq[lo:lo + nsp * sb], vis[j])

    for _ in range(warmup):
        step()
    torch.cuda.synchronize()
    plan.set_timing(True)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    f_ms, x_ms, count = plan.get_timing()
    plan.check()
    scale = plan.scale()
    plan.close()
    del iq, vis
    torch.cuda.empty_cache()
    return ms, f_ms / max(count, 1), x_ms / max(count, 1), scale


def f16_peaks(mdt, dev):
    """Measured f16 tensor throughput on this GPU: tcgen05.mma kind::f16 with
    its operands resident in shared memory, in the X-engine's instruction
    shape (M128 N128, two CTAs per SM) and in the widest one (M128 N256, one
    CTA per SM), and a cuBLAS fp16 GEMM (torch.matmul, 8192^3); each the best
    of several runs on random operands."""
    import torch
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    _, n128 = mdt.tc_peak_f16(128, 2, iters=20000, reps=5, err=err)
    _, n256 = mdt.tc_peak_f16(256, 1, iters=20000, reps=5, err=err)
    if int(err.item()) != 0:
        raise RuntimeError("tc_peak_f16: a completion wait timed out")
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    a = torch.randn(8192, 8192, dtype=torch.float16, device=dev, generator=g)
    b = torch.randn(8192, 8192, dtype=torch.float16, device=dev, generator=g)
    for _ in range(3):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    best = float("inf")
    for _ in range(10):
        e0.record()
        torch.matmul(a, b)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    torch.cuda.empty_cache()
    return {"tcgen05_kind_f16_m128n128_2cta_per_sm": n128,
            "tcgen05_kind_f16_m128n256_1cta_per_sm": n256,
            "cublas_fp16_gemm_8192": 2.0 * 8192 ** 3 / (best * 1e-3) / 1e12,
            "unit": "TFLOP/s", "method": "best of several runs, random operands"}


def tensor_path_section(mdt, dev, steps):
    """c3_array256 (NE=256, Nch=1024, Ntaps=8, Nsp=8192): the f16 tensor-core
    path (tensor-core F-engine + tensor-core X-engine) over the full 8
    integrations, the exact int8 path over the same, and the plain FP32 path
    and the SIMT-FFT f16 F-engine over one integration, in antenna-samples/s,
    with each kernel's roofline."""
    c3 = mdt.configs.C3
    hbm, bf16, kind = peaks()
    pk = f16_peaks(mdt, dev)
    ms16, f16, x16, scale = measure_plan(mdt, c3, 1, dev, steps=steps, warmup=1)
    ms8, f8, x8, _ = measure_plan(mdt, c3, 3, dev, steps=max(1, steps // 2), warmup=1)
    c3_one = mdt.configs.small(c3, nint=1)
    ms32, f32, x32, _ = measure_plan(mdt, c3_one, 0, dev, steps=1, warmup=1)
    os.environ["MDT_FENGINE"] = "simt"
    try:
        _, fsimt, _, _ = measure_plan(mdt, c3_one, 1, dev, steps=1, warmup=1)
    finally:
        del os.environ["MDT_FENGINE"]
    ne, nch, nsp, ntaps = c3.nelements, c3.nchannels, c3.nspectra, c3.ntaps
    flops = 8.0 * ne * (ne + 1) / 2 * nsp * nch
    v16 = c3.antenna_samples() / (ms16 * 1e-3)
    v8 = c3.antenna_samples() / (ms8 * 1e-3)
    v32 = c3_one.antenna_samples() / (ms32 * 1e-3)
    x_tflops = flops / (x16 * 1e-3) / 1e12
    f_bytes = (nsp + ntaps - 1) * ne * nch * 2 + nch * ((nsp + 31) // 32) * ((ne + 15) // 16 * 16) * 128

    def fe(ms, traffic=None):
        gbs = f_bytes / (ms * 1e-3) / 1e9
        return {"ms_per_launch": ms, "gbs": gbs, "frac": gbs / hbm, "bound": "hbm",
                "algorithmic_bytes": f_bytes, "peak_source": kind + " hbm_gbs",
                "traffic": traffic}

    return {
        "workload": c3.name, "precision": "f16 operands, fp32 accumulate (tcgen05 kind::f16)",
        "value": v16, "unit": "antenna-samples/s", "ms_per_step": ms16,
        "integrations": c3.nint, "fp32_path_value": v32, "speedup_vs_fp32_path": v16 / v32,
        "xengine_tc": {"ms_per_launch": x16, "tflops": x_tflops, "peak": bf16,
                       "frac": x_tflops / bf16, "peak_source": kind + " bf16_tflops (dense)",
                       "frac_of_measured_kind_f16": x_tflops / pk["tcgen05_kind_f16_m128n128_2cta_per_sm"],
                       "algorithmic_flops": flops, "traffic": NCU_TRAFFIC_C3["xengine_tc"]},
        "f16_peaks": pk,
        "fengine_tc": fe(f16, NCU_TRAFFIC_C3["fengine_tc"]),
        "fengine_simt_fft": fe(fsimt),
        "int8_path": {"value": v8, "unit": "antenna-samples/s", "ms_per_step": ms8,
                      "speedup_vs_fp32_path": v8 / v32, "fengine_ms": f8, "xengine_ms": x8,
                      "precision": "int8 F-output, exact int32 sums (f16 MMAs over FP32-exact "
                                   "windows)"},
        "fp32_path": {"fengine_ms": f32, "xengine_ms": x32},
        "f16_scale": scale,
    }


def batch_section(mdt, dev, steps):
    """Configuration 4: 24 ragged jobs (ragged_jobs()) in one graph-captured
    batch (f16 tensor path), aggregate antenna-samples/s per graph replay."""
    import torch
    jobs = mdt.configs.ragged_jobs()
    shapes = [(j.nelements, j.nchannels, j.ntaps, j.nspectra) for j in jobs]
    batch = mdt.FxBatch(shapes)
    maxw, cost_order = batch.autotune()
    iqs, viss = [], []
    for j in jobs:
        total = j.nspectra + j.ntaps - 1
        iq = torch.empty(total * j.nelements * j.nchannels * 2, dtype=torch.int8, device=dev)
        tone = j.tone_q16()
        mdt.synth_iq(j.seed, j.nelements, j.nchannels, 0, total,
                     torch.from_numpy(j.sigma_q8()).to(dev), iq,
                     tone_q16=None if tone is None else torch.from_numpy(tone).to(dev))
        iqs.append(iq)
        viss.append(torch.empty(j.nchannels, j.nelements, j.nelements, dtype=torch.complex64,
                                device=dev))
    torch.cuda.synchronize()
    batch.execute(iqs, viss)  # capture + first replay
    batch.check()
    stream = torch.cuda.ExternalStream(batch.stream)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        batch.execute(iqs, viss)
    e1.record(stream)
    batch.check()
    ms = e0.elapsed_time(e1) / steps
    samples = sum(j.antenna_samples() for j in jobs)
    batch.close()
    del iqs, viss
    torch.cuda.empty_cache()
    return {"workload": "c4_ragged24", "jobs": len(jobs), "value": samples / (ms * 1e-3),
            "unit": "antenna-samples/s", "ms_per_step": ms, "autotuned_maxw": maxw,
            "cost_ordered_work": cost_order, "graph": True,
            "precision": "f16 operands, fp32 accumulate"}


def gaincal_section(mdt, dev, steps):
    """Configuration 5 (NE=64, Nch=512, Ntaps=4, Nsp=2048, 3-source sky,
    gains with amplitude U[0.8, 1.2] and phase U[-pi, pi] on the F-engine
    output): device time of one differentiable FX pass (forward plus the
    hand-written adjoints for gains and PFB taps, F-engine output
    recomputed), and per-antenna gain calibration by preconditioned gradient
    descent to the stated relative gain error."""
    import torch
    adj = importlib.import_module("mdt_fpga-gpu_pipeline_gb300.adjoint")
    c5 = mdt.configs.C5
    ne, nch, ntaps, nsp = c5.nelements, c5.nchannels, c5.ntaps, c5.nspectra

    def t(a):
        return torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    ssig, sdel = c5.sources()
    iq = torch.empty((nsp + ntaps - 1) * ne * nch * 2, dtype=torch.int8, device=dev)
    mdt.synth_iq(c5.seed, ne, nch, 0, nsp + ntaps - 1, t(c5.sigma_q8()), iq,
                 src_sigma_q8=t(ssig), src_delay=t(sdel))
    win = torch.empty(nch * ntaps, dtype=torch.float32, device=dev)
    mdt.window_hamming_sinc(nch, ntaps, win)
    rng = np.random.default_rng([c5.seed, 9])
    g_true = t((rng.uniform(0.8, 1.2, (nch, ne)) *
                np.exp(1j * rng.uniform(-np.pi, np.pi, (nch, ne)))).astype(np.complex64))
    with torch.no_grad():
        data = adj.fx_correlate(iq, win, g_true, ne, nch, ntaps, nsp)
        model = adj.fx_correlate(iq, win, torch.ones_like(g_true), ne, nch, ntaps, nsp)
    taps = win.clone().requires_grad_(True)
    gains = torch.ones_like(g_true).requires_grad_(True)

    def fb():
        V = adj.fx_correlate(iq, taps, gains, ne, nch, ntaps, nsp)
        V.backward(V.detach())  # grad(V) = V: the loss sum |V|^2 / 2
    for _ in range(2):
        fb()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    stream = torch.cuda.current_stream(dev)
    e0.record(stream)
    for _ in range(steps):
        fb()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / steps
    # warm-up: the first solver step pays PyTorch's one-time kernel setup for the
    # loss's complex indexing and its backward (seconds on a fresh process)
    adj.solve_gains(iq, win, data, model, ne, nch, ntaps, nsp, iters=2, tol=0.0, true_gains=g_true)
    torch.cuda.synchronize()
    t0 = time.time()
    g, hist = adj.solve_gains(iq, win, data, model, ne, nch, ntaps, nsp, iters=200, tol=1e-11,
                              true_gains=g_true)
    torch.cuda.synchronize()
    wall = time.time() - t0
    err = adj.gain_error(g, g_true)
    to_target = next((i for i, (_, e) in enumerate(hist) if e is not None and e <= 1e-4), None)
    return {"workload": c5.name, "fwd_bwd_ms": ms,
            "fwd_bwd_value": c5.antenna_samples() / (ms * 1e-3), "unit": "antenna-samples/s",
            "gradients": "gains and PFB taps (adjoint kernels), F-output recomputed",
            "calibration_steps": len(hist), "steps_to_1e-4": to_target,
            "calibration_ms_per_step": wall / max(len(hist), 1) * 1e3,
            "gain_rel_error": err, "target_gain_rel_error": 1e-4}


def run_ours(args, cfg):
    import torch
    mdt = load_pkg()
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    mdt.lib()
    ne, nch, ntaps, nsp, nint = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra, cfg.nint
    sb = ne * nch * 2
    total_sp = nint * nsp + ntaps - 1
    dev = torch.device("cuda", local)

    def t(a):
        return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).to(dev)

    # replicas only: rank r takes integrations [r*nint, (r+1)*nint) of one
    # stream and generates just its span (the generator is counter-based)
    replicas = importlib.import_module("mdt_fpga-gpu_pipeline_gb300.replicas")
    first_int, _ = replicas.integration_split(nint * world, rank, world)
    s0, span = replicas.input_span(first_int, nint, nsp, ntaps)
    assert span == total_sp
    iq = torch.empty(total_sp * sb, dtype=torch.int8, device=dev)
    ssig, sdel = cfg.sources()
    mdt.synth_iq(cfg.seed, ne, nch, s0, total_sp, t(cfg.sigma_q8()), iq,
                 tone_q16=t(cfg.tone_q16()), src_sigma_q8=t(ssig), src_delay=t(sdel))
    win = torch.empty(nch * ntaps, dtype=torch.float32, device=dev)
    mdt.window_hamming_sinc(nch, ntaps, win)
    vis = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)
    prec = {"fp32": 0, "fp16": 1, "bf16": 2, "int8": 3}[args.precision]
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=prec, stream=stream)
    plan.set_window(win)

    first = (nsp + ntaps - 1) * sb

    def step():
        plan.stream_reset()
        plan.stream_push(iq[:first], vis[0])
        for j in range(1, nint):
            lo = (j * nsp + ntaps - 1) * sb
            plan.stream_push(iq[lo:lo + nsp * sb], vis[j])

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    for _ in range(args.warmup):
        step()
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    plan.set_timing(True)
    barrier()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    barrier()
    ms = e0.elapsed_time(e1) / args.steps
    clk = clocks.stop()
    f_ms, x_ms, count = plan.get_timing()
    plan.set_timing(False)
    if dist is not None:
        tt = torch.tensor([ms], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        ms = float(tt.item())
    samples = cfg.antenna_samples() * world
    value = samples / (ms * 1e-3)

    # ---- per-kernel roofline from the live kernel times (per launch)
    hbm, bf16, peak_kind = peaks()
    f_launch_ms = f_ms / max(count, 1)
    x_launch_ms = x_ms / max(count, 1)
    f_bytes = (nsp + ntaps - 1) * sb + nsp * ne * nch * 8 + ntaps * nch * 4
    x_flops = 8.0 * ne * (ne + 1) / 2 * nsp * nch
    x_bytes = nsp * ne * nch * 8 + nch * ne * ne * 8
    f_gbs = f_bytes / (f_launch_ms * 1e-3) / 1e9
    x_tflops = x_flops / (x_launch_ms * 1e-3) / 1e12
    x_gbs = x_bytes / (x_launch_ms * 1e-3) / 1e9
    sm_mhz = clk.get("sm_mhz") or 1900.0
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = nsm * 128 * 2 * sm_mhz * 1e6 / 1e12  # FP32 FMA lanes at the sampled clock
    if args.precision == "fp32":
        fname, xname, xbound, xpeak = "fengine_c64b", "xengine_herm_f32", "fp32", fp32_peak
        xpeak_src = ("nominal FP32 FMA rate (%d SMs x 128 lanes x 2) at the sampled SM clock"
                     % nsm)
    else:
        nep, nkc = (ne + 15) // 16 * 16, (nsp + 31) // 32
        f_bytes = (nsp + ntaps - 1) * sb + nch * nkc * nep * 128 + ntaps * nch * 4
        f_gbs = f_bytes / (f_launch_ms * 1e-3) / 1e9
        x_bytes = nch * nkc * nep * 128 + nch * ne * ne * 8
        x_gbs = x_bytes / (x_launch_ms * 1e-3) / 1e9
        ftc = nch == 1024 and ntaps in (4, 8)  # the tensor-core F-engine's shapes
        fname, xname, xbound, xpeak = ("fengine_tc" if ftc else "fengine_x16"), "xengine_tc", \
            "tensor", bf16
        xpeak_src = peak_kind + " bf16_tflops (dense, burst)"
    kernels = {
        fname: {"ms_per_launch": f_launch_ms, "bound": "hbm", "achieved": f_gbs, "unit": "GB/s",
                "peak": hbm, "frac": f_gbs / hbm, "algorithmic_bytes": f_bytes},
        xname: {"ms_per_launch": x_launch_ms, "bound": xbound, "achieved": x_tflops,
                "unit": "TFLOP/s", "peak": xpeak, "frac": x_tflops / xpeak,
                "algorithmic_flops": x_flops, "hbm_gbs": x_gbs},
    }
    if f_launch_ms >= x_launch_ms:
        roof = {"kernel": fname, "bound": "hbm", "achieved": f_gbs, "peak": hbm, "unit": "GB/s",
                "frac": f_gbs / hbm, "traffic": NCU_TRAFFIC.get(fname),
                "peak_source": peak_kind + " hbm_gbs"}
    else:
        roof = {"kernel": xname, "bound": xbound, "achieved": x_tflops, "peak": xpeak,
                "unit": "TFLOP/s", "frac": x_tflops / xpeak, "traffic": NCU_TRAFFIC.get(xname),
                "peak_source": xpeak_src}

    # ---- e2e through the host-buffer C-ABI entry (pinned host memory)
    e2e = None
    if not args.no_e2e:
        all_cpus = os.sched_getaffinity(0)
        host_cpus = bind_to_gpu_cpus(local)
        h_iq = torch.empty(total_sp * sb, dtype=torch.int8, pin_memory=True)
        h_iq.copy_(iq)
        h_vis = torch.empty(nint * nch * ne * ne * 2, dtype=torch.float32, pin_memory=True)
        plan.execute_host(h_iq, nint, h_vis)  # warm-up: staging buffers
        # each step timed on its own (execute_host returns after its last copy); the
        # median is reported, min and max beside it: the host link is shared with
        # other work on the machine and single steps can stall
        e2e_steps = max(3, min(args.steps, 7))
        barrier()
        times = []
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            plan.execute_host(h_iq, nint, h_vis)
            times.append(time.perf_counter() - t0)
        barrier()
        times.sort()
        e2e_s = times[len(times) // 2]
        if dist is not None:
            tt = torch.tensor([e2e_s], device=dev)
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            e2e_s = float(tt.item())
        # host result agrees with the device-resident run of the same stream
        ok = torch.equal(h_vis.view(torch.int32).view(-1).cpu(),
                         vis.view(torch.float32).view(torch.int32).view(-1).cpu())
        e2e = {"value": samples / e2e_s, "unit": "antenna-samples/s",
               "h2d_bytes_per_step": int(h_iq.numel()),
               "d2h_bytes_per_step": int(h_vis.numel() * 4),
               "api": "mdt_fx_execute_host", "matches_device_run": bool(ok),
               "host_cpus": host_cpus, "steps": e2e_steps, "statistic": "median step",
               "ms_per_step_min": times[0] * 1e3, "ms_per_step_max": times[-1] * 1e3}
        os.sched_setaffinity(0, all_cpus)  # the CPU baseline uses every core

    tensor = None
    if not args.no_tensor:
        tensor = tensor_path_section(mdt, dev, steps=max(1, min(args.steps, 3)))
    batched = None
    if not args.no_batch:
        batched = batch_section(mdt, dev, steps=max(1, min(args.steps, 5)))
    gaincal = None
    if not args.no_batch:
        gaincal = gaincal_section(mdt, dev, steps=max(1, min(args.steps, 10)))

    line = None
    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            rate, sample, cores, _ = cpu_pipeline_rate(cfg, args.cpu_budget)
            cpu = {"value": rate, "unit": "antenna-samples/s", "cores": cores, "kind": "port",
                   "sample": sample}
        line = {
            "metric": "F+X engine antenna-samples/s", "value": value, "unit": "antenna-samples/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp32": "f32", "fp16": "f16 operands / f32 accumulate",
                      "bf16": "bf16 operands / f32 accumulate",
                      "int8": "int8 F-output / exact int32 sums"}[args.precision],
            "data": "synthetic (seeded integer int8 I/Q generator)",
            "config": {"workload": cfg.name, "nelements": ne, "nchannels": nch, "ntaps": ntaps,
                       "nspectra": nsp, "integrations": nint,
                       "path": "fused plan API, %s" % args.precision,
                       "l2": "inputs (%.1f GB) larger than L2, no flush" % (iq.numel() / 1e9)},
            "e2e": e2e,
            "gpu_launches": 2 * nint * args.steps,
            "roofline": roof,
            "kernels": kernels,
            "cpu_baseline": cpu,
            "clocks": clk,
            "tensor_path": tensor,
            "batched": batched,
            "differentiation": gaincal,
        }
        print(json.dumps(line))
    plan.close()
    if dist is not None:
        dist.destroy_process_group()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="c2_station40")
    ap.add_argument("--cpu-budget", type=float, default=10.0,
                    help="seconds of CPU work for the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer e2e run")
    ap.add_argument("--no-batch", action="store_true", help="skip the c4 ragged-batch section")
    ap.add_argument("--no-tensor", action="store_true",
                    help="skip the c3 tensor-core vs FP32 section")
    ap.add_argument("--precision", choices=["fp32", "fp16", "bf16", "int8"], default="fp32",
                    help="plan precision of the main measurement")
    ap.add_argument("--nspectra", type=int, default=None,
                    help="override spectra per integration (small profiling cases)")
    ap.add_argument("--integrations", type=int, default=None,
                    help="override the number of integrations per step (small profiling "
                         "cases)")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours":
        print("warning: fewer than 3 warm-up steps", file=sys.stderr)
    mdt = load_pkg()
    cfg = mdt.configs.CONFIGS[args.config]
    if args.integrations:
        cfg = mdt.configs.small(cfg, nint=args.integrations)
    if args.nspectra:
        cfg = mdt.configs.small(cfg, nspectra=args.nspectra)
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_ours(args, cfg)


if __name__ == "__main__":
    main()

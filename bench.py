#!/usr/bin/env python
"""Benchmark of the FX correlator hot path on one GB300 (or N replicas).

Workload (default): c3_array256 -- NE=256 inputs, Nch=1024, Ntaps=8,
Nspectra=8192, 8 integrations streamed back to back with the PFB history
carried between them; synthetic int8 I/Q from the integer generator (3 point
sources with geometric delays in unit receiver noise at SNR 0.1).  One step =
the 8 integrations through the plan API on the f16 tensor-core path
(tensor-core F-engine -> tcgen05 Hermitian X-engine, FP32 accumulation).
Metric: antenna-samples/s = NE * Nspectra * Nch * 8 / step time.  The 34.4 GB
input stream is larger than L2, so no L2 flush is needed between steps.

  value         device-timed (CUDA events on the plan's stream), inputs resident
  e2e           same metric through mdt_fx_execute_host: pinned host samples
                in, host visibilities out, copies inside the timed region
  roofline      the dominant kernel, achieved from live CUDA-event kernel times
  accuracy      relative visibility error against the FP64 oracle (a checker,
                run after the timed regions) on a channel subset of the first
                timed integration, for every precision; int32 sums of the int8
                path checked bit for bit against the integer oracle
  cpu_baseline  the oracle's FP32 OpenMP pipeline on a bounded sample (rank 0)
Extra keys: the other precisions on the same stream and the plain FP32 path
(the >= 4x target's denominator), the host link's own bandwidth, the c2
station (FP32, 16 integrations), the library bar (the reference's own
kernels with cuFFT and cuBLAS, per integration), the c4 ragged batch and the
c5 differentiation and gain calibration.

--impl reference times the reference path's CPU implementation on the host
cores.  The reference has no CPU FX code, so this is the oracle port (FP32,
OpenMP, all host threads) on a bounded sample of the same workload.

Multi-GPU (torchrun): replicas only -- rank r runs integrations
[nint*r, nint*(r+1)) of one stream (its own span of the counter-based
generator, lead-in included), no data-path collective; value = all ranks'
samples / max rank time ("scaling": "weak").
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

PREC = {"fp32": 0, "fp16": 1, "bf16": 2, "int8": 3}
DTYPE = {"fp32": "f32", "fp16": "f16 operands / f32 accumulate",
         "bf16": "bf16 operands / f32 accumulate", "int8": "int8 F-output / exact int32 sums"}

# DRAM bytes (read + write) per launch from ncu captures (see profiles/).
# FP32 path on one c2 integration (profiles/fengine_c64b_c2.txt,
# profiles/xengine_herm_f32_c2.txt): the bench's launches are that integration.
NCU_TRAFFIC_C2 = {"fengine_c64b": 677.995e6 + 2637.297e6,
                  "xengine_herm_f32": 2684.435e6 + 26.480e6}
# Tensor path on one c3 integration (Nsp = 8192), scaled from captures at
# Nsp = 1024 (profiles/fengine_tc_c3.txt, profiles/xengine_tc_c3.txt): the
# F-engine's reads and writes and the X-engine's operand reads grow with the
# spectra processed, the X-engine's visibility writes do not.
NCU_TRAFFIC_C3 = {"fengine_tc": 0.544354e9 * 8199 / 1031 + 1.025016e9 * 8,
                  "xengine_tc": 1.075430e9 * 8 + 0.488982e9}


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


# ----------------------------------------------------------------- inputs
def t_dev(a, dev):
    import torch
    return None if a is None else torch.from_numpy(np.ascontiguousarray(a)).to(dev)


def make_stream(mdt, cfg, dev, s0, nspectra_total):
    """int8 I/Q of spectra s0 .. s0+nspectra_total-1 of the configuration's stream."""
    import torch
    sb = cfg.nelements * cfg.nchannels * 2
    iq = torch.empty(nspectra_total * sb, dtype=torch.int8, device=dev)
    ssig, sdel = cfg.sources()
    mdt.synth_iq(cfg.seed, cfg.nelements, cfg.nchannels, s0, nspectra_total,
                 t_dev(cfg.sigma_q8(), dev), iq, tone_q16=t_dev(cfg.tone_q16(), dev),
                 src_sigma_q8=t_dev(ssig, dev), src_delay=t_dev(sdel, dev))
    return iq


def make_window(mdt, cfg, dev):
    import torch
    win = torch.empty(cfg.nchannels * cfg.ntaps, dtype=torch.float32, device=dev)
    mdt.window_hamming_sinc(cfg.nchannels, cfg.ntaps, win)
    return win


def stream_steps(plan, iq, vis, cfg):
    """One step: the configuration's integrations pushed through the plan."""
    sb = cfg.nelements * cfg.nchannels * 2
    nsp, ntaps = cfg.nspectra, cfg.ntaps
    first = (nsp + ntaps - 1) * sb

    def step():
        plan.stream_reset()
        plan.stream_push(iq[:first], vis[0])
        for j in range(1, cfg.nint):
            lo = (j * nsp + ntaps - 1) * sb
            plan.stream_push(iq[lo:lo + nsp * sb], vis[j])
    return step


def measure_plan(mdt, cfg, precision, dev, steps, warmup, iq=None, win=None):
    """Device-timed streamed FX over cfg.nint integrations with the plan API.
    Returns (ms per step, F-engine ms per launch, X-engine ms per launch,
    plan scale)."""
    import torch
    own = iq is None
    if own:
        iq = make_stream(mdt, cfg, dev, 0, cfg.total_spectra())
    if win is None:
        win = make_window(mdt, cfg, dev)
    ne, nch = cfg.nelements, cfg.nchannels
    vis = torch.empty(cfg.nint, nch, ne, ne, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)
    plan = mdt.FxPlan(ne, nch, cfg.ntaps, cfg.nspectra, precision=precision, stream=stream)
    plan.set_window(win)
    step = stream_steps(plan, iq, vis, cfg)
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
    del vis
    if own:
        del iq
    torch.cuda.empty_cache()
    return ms, f_ms / max(count, 1), x_ms / max(count, 1), scale


def kernel_roofline(cfg, precision, f_ms, x_ms, sm_mhz, nsm, fp32_peak=None):
    """Per-kernel figures of one integration: (kernels dict, roofline of the
    slower one).  Bytes per launch: F-engine reads 2 B per input sample
    (Nsp + Ntaps - 1 spectra) and writes its output layout (8 B per sample
    complex64, or the tensor operand rows: 128 B per (32 spectra, channel,
    padded element)); X-engine flops 8 * NE(NE+1)/2 * Nsp * Nch."""
    hbm, bf16, peak_kind = peaks()
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    sb = ne * nch * 2
    x_flops = 8.0 * ne * (ne + 1) / 2 * nsp * nch
    if precision == "fp32":
        f_bytes = (nsp + ntaps - 1) * sb + nsp * ne * nch * 8 + ntaps * nch * 4
        x_bytes = nsp * ne * nch * 8 + nch * ne * ne * 8
        fname, xname, xbound = "fengine_c64b", "xengine_herm_f32", "fp32"
        xpeak = nsm * 128 * 2 * (sm_mhz or 1900.0) * 1e6 / 1e12
        xpeak_src = ("nominal FP32 FMA rate (%d SMs x 128 lanes x 2) at the sampled SM clock"
                     % nsm)
        if fp32_peak:
            xpeak = fp32_peak
            xpeak_src = ("measured FP32 FMA rate (mdt_fp32_peak: one 1024-thread CTA per SM, "
                         "independent FMA chains, the faster of packed f32x2 and scalar)")
        traffic = NCU_TRAFFIC_C2 if cfg.name == "c2_station40" else {}
    else:
        nep, nkc = (ne + 15) // 16 * 16, (nsp + 31) // 32
        f_bytes = (nsp + ntaps - 1) * sb + nch * nkc * nep * 128 + ntaps * nch * 4
        x_bytes = nch * nkc * nep * 128 + nch * ne * ne * 8
        ftc = nch == 1024 and ntaps in (4, 8)  # the tensor-core F-engine's shapes
        fname = "fengine_tc" if ftc else ("fengine_q8" if precision == "int8" else "fengine_x16")
        xname, xbound, xpeak = ("xengine_q8" if precision == "int8" else "xengine_tc"), \
            "tensor", bf16
        xpeak_src = peak_kind + " bf16_tflops (dense, burst)"
        traffic = NCU_TRAFFIC_C3 if (cfg.name == "c3_array256" and precision in ("fp16", "bf16")) \
            else {}
    f_gbs = f_bytes / (f_ms * 1e-3) / 1e9
    x_tflops = x_flops / (x_ms * 1e-3) / 1e12
    kernels = {
        fname: {"ms_per_launch": f_ms, "bound": "hbm", "achieved": f_gbs, "unit": "GB/s",
                "peak": hbm, "frac": f_gbs / hbm, "algorithmic_bytes": f_bytes,
                "traffic": traffic.get(fname)},
        xname: {"ms_per_launch": x_ms, "bound": xbound, "achieved": x_tflops,
                "unit": "TFLOP/s", "peak": xpeak, "frac": x_tflops / xpeak,
                "peak_source": xpeak_src, "algorithmic_flops": x_flops,
                "hbm_gbs": x_bytes / (x_ms * 1e-3) / 1e9, "traffic": traffic.get(xname)},
    }
    if f_ms >= x_ms:
        roof = {"kernel": fname, "bound": "hbm", "achieved": f_gbs, "peak": hbm, "unit": "GB/s",
                "frac": f_gbs / hbm, "traffic": traffic.get(fname),
                "peak_source": peak_kind + " hbm_gbs", "algorithmic_bytes_per_launch": f_bytes,
                "ms_per_launch": f_ms}
    else:
        roof = {"kernel": xname, "bound": xbound, "achieved": x_tflops, "peak": xpeak,
                "unit": "TFLOP/s", "frac": x_tflops / xpeak, "traffic": traffic.get(xname),
                "peak_source": xpeak_src, "algorithmic_flops_per_launch": x_flops,
                "ms_per_launch": x_ms}
    return kernels, roof


# ------------------------------------------------------------ CPU baseline
def cpu_pipeline_rate(cfg, budget_s, threads=None):
    """Oracle FP32 OpenMP pipeline on the host: (samples/s, sample text, cores,
    spectra).  The sample is the first spectra of one integration, all
    channels, sized to about `budget_s` seconds."""
    from oracle import oracle
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    ne, nch, ntaps = cfg.nelements, cfg.nchannels, cfg.ntaps
    cores = int(os.environ.get("OMP_NUM_THREADS", len(os.sched_getaffinity(0))))
    win = oracle.window_hamming_sinc(nch, ntaps)
    ssig, sdel = cfg.sources()

    def run(nsp):
        iq = oracle.synth_iq(cfg.seed, ne, nch, 0, nsp + ntaps - 1, cfg.sigma_q8(),
                             cfg.tone_q16(), ssig, sdel)
        t0 = time.perf_counter()
        oracle.fx(iq, win, ne, nch, ntaps, nsp, double=False)
        return time.perf_counter() - t0

    probe = 32
    dt = run(probe)
    nsp = int(max(32, min(cfg.nspectra, probe * budget_s / max(dt, 1e-3))))
    dt = run(nsp)
    rate = ne * nsp * nch / dt
    sample = ("%s shape (NE=%d, Nch=%d, Ntaps=%d), first %d of %d spectra of one integration, "
              "all channels, FP32 OpenMP oracle pipeline (F-engine rows, then Hermitian "
              "per-channel products)" % (cfg.name, ne, nch, ntaps, nsp, cfg.nspectra))
    return rate, sample, cores, nsp


def run_reference(args, cfg):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle
    oracle.build()
    ne, nch, ntaps = cfg.nelements, cfg.nchannels, cfg.ntaps
    cores = len(os.sched_getaffinity(0))
    win = oracle.window_hamming_sinc(nch, ntaps)
    ssig, sdel = cfg.sources()

    def inputs(nsp):
        return oracle.synth_iq(cfg.seed, ne, nch, 0, nsp + ntaps - 1, cfg.sigma_q8(),
                               cfg.tone_q16(), ssig, sdel)
    # size each step to ~3 s of CPU work
    iq = inputs(32)
    t0 = time.perf_counter()
    oracle.fx(iq, win, ne, nch, ntaps, 32, double=False)
    per_sp = (time.perf_counter() - t0) / 32
    nsp = int(max(32, min(cfg.nspectra, 3.0 / max(per_sp, 1e-6))))
    iq = inputs(nsp)
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
                "OpenMP restatement of its GPU sequence (F-engine rows, then Hermitian "
                "per-channel products) on all host threads",
    }
    print(json.dumps(line))


# --------------------------------------------------------------- accuracy
def accuracy_section(mdt, cfg, dev, iq, win, vis_main, main_precision, nsel=16):
    """Error of each precision against the FP64 oracle on a channel subset of
    the first integration of the timed stream (the oracle is the checker
    here, run after the timed regions).  The main precision is read from the
    timed run's own visibilities; the others are run on the same samples.
    For int8, the plan's stages are rerun with its calibrated channel scales
    to expose the int32 sums, which are compared bit for bit with the
    integer oracle on the same channels of the GPU's int8 F-output."""
    import torch
    from oracle import oracle
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    sb = ne * nch * 2
    first = (nsp + ntaps - 1) * sb
    sel = np.unique(np.concatenate([[0, 1, nch // 2, nch - 1],
                                    np.linspace(0, nch - 1, nsel).astype(np.int64)]))
    sel = sel.astype(np.int32)
    iq0 = iq[:first]
    iq0_h = iq0.cpu().numpy()
    t0 = time.time()
    ref = oracle.fx(iq0_h, win.cpu().numpy(), ne, nch, ntaps, nsp, channels=sel)
    oracle_s = time.time() - t0
    den = np.linalg.norm(ref.reshape(len(sel), -1), axis=1)

    def errs(v):
        d = (v[sel] - ref).reshape(len(sel), -1)
        fro = np.linalg.norm(d, axis=1) / den
        return {"rel_err_vs_fp64": float(fro.max()),
                "max_abs_err_over_max_abs": float(np.abs(d).max() / np.abs(ref).max())}

    out = {"channels": sel.tolist(), "integration": 0,
           "statistic": "max over the channels of ||V - V_fp64||_F / ||V_fp64||_F",
           "oracle": "FP64 restatement of PpS_Batch -> FFT -> reorder -> CGEMM, %.1f s" % oracle_s}
    tol = {"fp32": 1e-5, "fp16": 1e-3, "bf16": 4e-3, "int8": 2e-2}
    for prec in ("fp16", "bf16", "fp32", "int8"):
        if prec == main_precision:
            v = vis_main[0].cpu().numpy()
            src = "the timed run"
        else:
            plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=PREC[prec])
            plan.set_window(win)
            vis = torch.empty(nch, ne, ne, dtype=torch.complex64, device=dev)
            plan.execute(iq0, 1, vis)
            plan.check()
            if prec == "int8":
                qs = torch.empty(nch, dtype=torch.float32, device=dev)
                plan.get_channel_scales(qs)
            plan.close()
            v = vis.cpu().numpy()
            del vis
            src = "one plan integration on the same samples"
        e = errs(v)
        e["tolerance"] = tol[prec]
        e["within_tolerance"] = e["rel_err_vs_fp64"] <= tol[prec]
        e["source"] = src
        if prec == "int8":
            e.update(int8_exactness(mdt, cfg, dev, iq0, win, qs, v, sel))
        out[prec] = e
        torch.cuda.empty_cache()
    return out


def int8_exactness(mdt, cfg, dev, iq0, win, qs, vis_plan, sel):
    import torch
    from oracle import oracle
    ne, nch, ntaps, nsp = cfg.nelements, cfg.nchannels, cfg.ntaps, cfg.nspectra
    nep, nkc = (ne + 15) // 16 * 16, (nsp + 31) // 32
    X16 = torch.zeros(mdt.x16_bytes(ne, nch, nsp), dtype=torch.uint8, device=dev)
    err = torch.zeros(1, dtype=torch.int32, device=dev)
    if nch == 1024 and ntaps in (4, 8):
        mdt.fengine_tc_q8(ne, nch, ntaps, nsp, iq0, win, X16, qs, err)
        fe = "fengine_tc (int8 requantised output)"
    else:
        mdt.fengine_q8(ne, nch, ntaps, nsp, iq0, win, X16, qs)
        fe = "fengine_q8"
    raw = torch.empty(nch, ne, ne, 2, dtype=torch.int32, device=dev)
    vis = torch.empty(nch, ne, ne, dtype=torch.complex64, device=dev)
    mdt.xengine_q8(ne, nch, nsp, X16, qs, vis=vis, vis_i32=raw, err=err)
    torch.cuda.synchronize()
    same_as_plan = bool(np.array_equal(vis.cpu().numpy().view(np.int64),
                                       vis_plan.view(np.int64)))
    # the selected channels of the int8 F-output, decoded from the operand rows
    rows = X16.view(nkc, nch, nep, 64 * 2)[:, torch.from_numpy(sel.astype(np.int64)).to(dev)]
    rows = rows.cpu().numpy().view(np.float16).reshape(nkc, len(sel), nep, 64)
    L = np.arange(64)
    X = np.zeros((len(sel), nkc * 32, ne, 2), np.float32)
    for e in range(ne):
        p = (((L >> 3) ^ (e & 7)) << 3) | (L & 7)
        lg = rows[:, :, e, :][:, :, p].transpose(1, 0, 2)  # [k][kc][64]
        X[:, :, e, 0] = lg[:, :, :32].reshape(len(sel), -1)
        X[:, :, e, 1] = lg[:, :, 32:].reshape(len(sel), -1)
    X = X[:, :nsp]
    integral = bool(np.all(X == np.rint(X)) and np.abs(X).max() <= 127)
    ref = oracle.xengine_i8(X.astype(np.int8), ne, len(sel), nsp)
    got = raw[torch.from_numpy(sel.astype(np.int64)).to(dev)].cpu().numpy().astype(np.int64)
    return {"int32_bit_exact": bool(np.array_equal(got, ref)) and integral,
            "int32_check": "int32 sums of xengine_q8 on the plan's scales vs the integer "
                           "oracle on the same channels of the GPU's int8 F-output (%s); the "
                           "stage rerun equals the plan's visibilities bit for bit: %s"
                           % (fe, same_as_plan)}


# --------------------------------------------------------------- sections
def link_section(dev, gib=4):
    """The host link's own bandwidth: pinned host <-> device copies of `gib`
    GiB (one cudaMemcpyAsync each), best of 3, CUDA events."""
    import torch
    n = gib << 30
    h = torch.empty(n, dtype=torch.uint8, pin_memory=True)
    h.fill_(1)
    d = torch.empty(n, dtype=torch.uint8, device=dev)
    s = torch.cuda.current_stream(dev)
    res = {}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        best = float("inf")
        for _ in range(3):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(s)
            dst.copy_(src, non_blocking=True)
            e1.record(s)
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1))
        res[name] = n / (best * 1e-3) / 1e9
    del h, d
    torch.cuda.empty_cache()
    res["bytes"] = n
    res["method"] = "pinned host buffer, one cudaMemcpyAsync, best of 3"
    return res


def e2e_run(mdt, cfg, precision, dev, iq, vis_dev, samples, steps, barrier, local):
    """Same workload through mdt_fx_execute_host from pinned host memory."""
    import torch
    ne, nch = cfg.nelements, cfg.nchannels
    all_cpus = os.sched_getaffinity(0)
    host_cpus = bind_to_gpu_cpus(local)
    h_iq = torch.empty(iq.numel(), dtype=torch.int8, pin_memory=True)
    h_iq.copy_(iq)
    h_vis = torch.empty(cfg.nint * nch * ne * ne * 2, dtype=torch.float32, pin_memory=True)
    win = make_window(mdt, cfg, dev)
    plan = mdt.FxPlan(ne, nch, cfg.ntaps, cfg.nspectra, precision=PREC[precision])
    plan.set_window(win)
    plan.execute_host(h_iq, cfg.nint, h_vis)  # warm-up: staging buffers
    barrier()
    # each step timed on its own (execute_host returns after its last copy);
    # the median is reported, min and max beside it
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        plan.execute_host(h_iq, cfg.nint, h_vis)
        times.append(time.perf_counter() - t0)
    barrier()
    plan.check()
    plan.close()
    ok = None
    if vis_dev is not None:
        ok = torch.equal(h_vis.view(torch.int32).view(-1).cpu(),
                         vis_dev.view(torch.float32).view(torch.int32).view(-1).cpu())
    srt = sorted(times)
    res = {"median_s": srt[len(srt) // 2], "api": "mdt_fx_execute_host",
           "h2d_bytes_per_step": int(h_iq.numel()), "d2h_bytes_per_step": int(h_vis.numel() * 4),
           "matches_device_run": None if ok is None else bool(ok), "host_cpus": host_cpus,
           "steps": steps, "statistic": "median step",
           "ms_per_step_min": srt[0] * 1e3, "ms_per_step_max": srt[-1] * 1e3,
           "ms_per_step_all": [round(x * 1e3, 2) for x in times]}
    os.sched_setaffinity(0, all_cpus)  # the CPU baseline uses every core
    del h_iq, h_vis
    return res


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
    dev = torch.device("cuda", local)
    precision = args.precision

    # replicas only: rank r takes integrations [r*nint, (r+1)*nint) of one
    # stream and generates just its span (the generator is counter-based)
    replicas = importlib.import_module("mdt_fpga-gpu_pipeline_gb300.replicas")
    first_int, _ = replicas.integration_split(nint * world, rank, world)
    s0, span = replicas.input_span(first_int, nint, nsp, ntaps)
    assert span == cfg.total_spectra()
    iq = make_stream(mdt, cfg, dev, s0, span)
    win = make_window(mdt, cfg, dev)
    vis = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, precision=PREC[precision], stream=stream)
    plan.set_window(win)
    step = stream_steps(plan, iq, vis, cfg)

    def barrier():
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()

    def max_over_ranks(x):
        if dist is None:
            return x
        tt = torch.tensor([x], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        return float(tt.item())

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
    plan.check()
    plan.close()
    ms = max_over_ranks(ms)
    samples = cfg.antenna_samples() * world
    value = samples / (ms * 1e-3)
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    kernels, roof = kernel_roofline(cfg, precision, f_ms / max(count, 1), x_ms / max(count, 1),
                                    clk.get("sm_mhz"), nsm)

    e2e = None
    if not args.no_e2e:
        r = e2e_run(mdt, cfg, precision, dev, iq, vis, samples / world,
                    max(3, min(args.steps, 10)), barrier, local)
        e2e_s = max_over_ranks(r.pop("median_s"))
        e2e = {"value": samples / e2e_s, "unit": "antenna-samples/s"}
        e2e.update(r)

    extras = {}
    want = set()
    if not args.no_extras:
        want = set(("accuracy,paths,link,station_c2,library_bar,batched,differentiation"
                    if args.sections == "all" else args.sections).split(","))
    if rank == 0 and "accuracy" in want:
        extras["accuracy"] = accuracy_section(mdt, cfg, dev, iq, win, vis, precision)
    del vis
    torch.cuda.empty_cache()
    if "paths" in want:
        extras.update(paths_section(mdt, cfg, dev, iq, win, ms, precision,
                                    max(1, min(args.steps, 3))))
    del iq
    torch.cuda.empty_cache()
    if "link" in want:
        extras["link"] = link_section(dev)
        if e2e is not None:
            h2d = extras["link"]["h2d_gbs"]
            e2e["link_floor_value"] = samples / (e2e["h2d_bytes_per_step"] / (h2d * 1e9))
            e2e["link_note"] = ("inputs alone at the link's measured H2D rate; e2e is "
                                "link-bound when value is near this")
    if "station_c2" in want:
        extras["station_c2"] = station_section(mdt, dev, max(1, min(args.steps, 5)), barrier,
                                               local, not args.no_e2e)
    if "library_bar" in want:
        extras["library_bar"] = library_bar_section(mdt, dev)
    if "batched" in want:
        extras["batched"] = batch_section(mdt, dev, steps=max(1, min(args.steps, 5)))
    if "differentiation" in want:
        extras["differentiation"] = gaincal_section(mdt, dev, steps=max(1, min(args.steps, 10)))

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
            "dtype": DTYPE[precision],
            "data": "synthetic (seeded integer int8 I/Q generator)",
            "config": {"workload": cfg.name, "nelements": ne, "nchannels": nch, "ntaps": ntaps,
                       "nspectra": nsp, "integrations": nint, "precision": precision,
                       "path": "fused plan API (tensor-core F-engine and X-engine)"
                               if precision != "fp32" else "fused plan API, FP32",
                       "l2": "inputs (%.1f GB) larger than L2, no flush" %
                             (cfg.total_spectra() * ne * nch * 2 / 1e9)},
            "e2e": e2e,
            "gpu_launches": 2 * nint * args.steps,
            "roofline": roof,
            "kernels": kernels,
            "cpu_baseline": cpu,
            "clocks": clk,
        }
        line.update(extras)
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return line


def paths_section(mdt, cfg, dev, iq, win, main_ms, main_precision, steps):
    """The other precisions on the same stream over all integrations, the
    plain FP32 path (the >= 4x target's denominator) and the SIMT-FFT f16
    F-engine over one integration, the measured f16 tensor peaks, and the
    speed-up of each path over the FP32 path."""
    samples = cfg.antenna_samples()
    res = {}
    for prec in ("fp16", "bf16", "int8"):
        if prec == main_precision:
            continue
        ms, f, x, _ = measure_plan(mdt, cfg, PREC[prec], dev, steps=steps, warmup=1, iq=iq,
                                   win=win)
        res[prec + "_path"] = {"value": samples / (ms * 1e-3), "unit": "antenna-samples/s",
                               "ms_per_step": ms, "fengine_ms": f, "xengine_ms": x,
                               "precision": DTYPE[prec]}
    one = load_pkg().configs.small(cfg, nint=1)
    sb = cfg.nelements * cfg.nchannels * 2
    iq1 = iq[:one.total_spectra() * sb]
    ms32, f32, x32, _ = measure_plan(mdt, one, 0, dev, steps=2, warmup=1, iq=iq1, win=win)
    v32 = one.antenna_samples() / (ms32 * 1e-3)
    res["fp32_path"] = {"value": v32, "unit": "antenna-samples/s", "ms_per_integration": ms32,
                        "fengine_ms": f32, "xengine_ms": x32,
                        "note": "one integration of the same stream (the X-engine is FP32 "
                                "SIMT; its speed does not depend on the integration)"}
    main_value = samples / (main_ms * 1e-3)
    res["speedup_vs_fp32_path"] = {main_precision: main_value / v32}
    for k in ("fp16", "bf16", "int8"):
        if k + "_path" in res:
            res["speedup_vs_fp32_path"][k] = res[k + "_path"]["value"] / v32
    if main_precision != "fp32" and cfg.nchannels == 1024:
        os.environ["MDT_FENGINE"] = "simt"
        try:
            _, fsimt, _, _ = measure_plan(mdt, one, PREC[main_precision], dev, steps=2, warmup=1,
                                          iq=iq1, win=win)
        finally:
            del os.environ["MDT_FENGINE"]
        res["fengine_simt_fft_ms"] = fsimt
    if main_precision != "fp32":
        res["f16_peaks"] = f16_peaks(mdt, dev)
    return res


def station_section(mdt, dev, steps, barrier, local, with_e2e):
    """c2_station40 (NE=40, Nch=2048, Ntaps=8, Nsp=4096, 16 integrations) on
    the plain FP32 path: device-timed, per-kernel roofline and e2e."""
    import torch
    c2 = mdt.configs.C2
    iq = make_stream(mdt, c2, dev, 0, c2.total_spectra())
    win = make_window(mdt, c2, dev)
    ms, f, x, _ = measure_plan(mdt, c2, 0, dev, steps=steps, warmup=2, iq=iq, win=win)
    nsm = torch.cuda.get_device_properties(dev).multi_processor_count
    _, fp32_packed = mdt.fp32_peak(True)
    _, fp32_scalar = mdt.fp32_peak(False)
    kernels, roof = kernel_roofline(c2, "fp32", f, x, 2070.0, nsm,
                                    fp32_peak=max(fp32_packed, fp32_scalar))
    res = {"workload": c2.name, "precision": "fp32", "value": c2.antenna_samples() / (ms * 1e-3),
           "unit": "antenna-samples/s", "ms_per_step": ms, "integrations": c2.nint,
           "kernels": kernels, "roofline": roof,
           "fp32_peaks": {"fma_f32x2": fp32_packed, "fma_f32": fp32_scalar,
                          "nominal": nsm * 128 * 2 * 2070.0e6 / 1e12, "unit": "TFLOP/s"}}
    if with_e2e:
        r = e2e_run(mdt, c2, "fp32", dev, iq, None, c2.antenna_samples(), 5, barrier, local)
        res["e2e"] = {"value": c2.antenna_samples() / r.pop("median_s"),
                      "unit": "antenna-samples/s", **r}
    del iq
    torch.cuda.empty_cache()
    return res


def library_bar_section(mdt, dev):
    """The reference's own GPU sequence per integration (its PpS_Batch and
    ReorderFOutput compiled from the reference source, cuFFT, cuBLAS
    CgemmBatched, the history copy), at c2 and c3, next to this library's
    FP32 path and tensor path on the same integration."""
    import torch
    from baseline import refseq
    if not refseq.available():
        return {"unavailable": "reference kernels not compiled (baseline/build_ref_gpu.sh)"}
    fft_file, blas_file, fft_ver, blas_ver = refseq.libraries()
    out = {"what": "reference kernels (sm_103a build of MDT_device_functions.cu) + cuFFT + "
                   "cuBLAS, launched as MDT_OneStation_client.cu:1083-1170 does, one "
                   "integration per rep; complex64 input converted exactly from the int8 I/Q",
           "libraries": {"cufft": fft_file, "cufft_version": fft_ver, "cublas": blas_file,
                         "cublas_version": blas_ver}}
    for cfg, tensor_prec in ((mdt.configs.C2, None), (mdt.configs.C3, "fp16")):
        one = mdt.configs.small(cfg, nint=1)
        ne, nch, ntaps, nsp = one.nelements, one.nchannels, one.ntaps, one.nspectra
        iq = make_stream(mdt, one, dev, 0, one.total_spectra())
        win = make_window(mdt, one, dev)
        ours32, f32, x32, _ = measure_plan(mdt, one, 0, dev, steps=3, warmup=1, iq=iq, win=win)
        entry = {"fp32_path_ms": ours32}
        if tensor_prec:
            ms16, _, _, _ = measure_plan(mdt, one, PREC[tensor_prec], dev, steps=3, warmup=1,
                                         iq=iq, win=win)
            entry["tensor_path_ms"] = ms16
        torch.cuda.empty_cache()
        try:
            rs = refseq.RefSeq(ne, nch, ntaps, nsp)
            try:
                rs.set_input(iq, win)
                rs.run(1)
                stages, total = rs.run(3)
            finally:
                rs.close()
            entry.update({"reference_ms_per_integration": total, "reference_stages_ms": stages,
                          "fp32_path_speedup": total / ours32})
            if tensor_prec:
                entry["tensor_path_speedup"] = total / entry["tensor_path_ms"]
        except refseq.RefSeqError as e:
            entry["unavailable"] = str(e)
        del iq
        torch.cuda.empty_cache()
        out[cfg.name] = entry
    return out


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
        iqs.append(make_stream(mdt, j, dev, 0, j.nspectra + j.ntaps - 1))
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
    """Configuration 5 (NE=64, Nch=512, Ntaps=4, Nsp=2048): device time of one
    differentiable FX pass (forward plus the hand-written adjoints for gains
    and PFB taps, F-engine output recomputed), and per-antenna gain
    calibration of the noisy, gained sky against the independent source
    model (the noise-free source streams' correlation) by preconditioned
    gradient descent: the error against the true gains (limited by the
    receiver noise) and against the loss minimiser (the solver's own
    convergence)."""
    import torch
    adj = importlib.import_module("mdt_fpga-gpu_pipeline_gb300.adjoint")
    c5 = mdt.configs.C5
    ne, nch, ntaps, nsp = c5.nelements, c5.nchannels, c5.ntaps, c5.nspectra
    win = make_window(mdt, c5, dev)
    data, iq_model, model, g_true = adj.c5_calibration_inputs(mdt, c5, win)
    taps = win.clone().requires_grad_(True)
    gains = torch.ones_like(g_true).requires_grad_(True)

    def fb():
        V = adj.fx_correlate(iq_model, taps, gains, ne, nch, ntaps, nsp)
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
    # warm-up: the first solver step pays PyTorch's one-time kernel setup
    adj.solve_gains(iq_model, win, data, model, ne, nch, ntaps, nsp, iters=2, tol=0.0,
                    true_gains=g_true)
    torch.cuda.synchronize()
    t0 = time.time()
    g, hist = adj.solve_gains(iq_model, win, data, model, ne, nch, ntaps, nsp, iters=400,
                              tol=1e-13, gtol=1e-7, true_gains=g_true)
    torch.cuda.synchronize()
    wall = time.time() - t0
    g_min, _ = adj.solve_gains(iq_model, win, data, model, ne, nch, ntaps, nsp, iters=400,
                               tol=1e-13, gtol=1e-7, g0=g_true)
    err = adj.gain_error(g, g_true)
    return {"workload": c5.name, "fwd_bwd_ms": ms,
            "fwd_bwd_value": c5.antenna_samples() / (ms * 1e-3), "unit": "antenna-samples/s",
            "gradients": "gains and PFB taps (adjoint kernels), F-output recomputed",
            "model": "correlation of the noise-free source streams (known flux and delays), "
                     "independent of the receiver noise in the data",
            "calibration_steps": len(hist), "calibration_ms_per_step": wall / len(hist) * 1e3,
            "gain_rel_error_vs_true": err,
            "gain_rel_error_vs_loss_minimiser": adj.gain_error(g, g_min),
            "noise_floor_gain_error": adj.gain_error(g_min, g_true),
            "start_gain_rel_error": hist[0][1], "final_rel_loss": hist[-1][0],
            "target_gain_rel_error": 1e-4,
            "note": "at SNR 0.1 and 2048 spectra the receiver noise limits the gains to the "
                    "noise floor above; the solver reaches the loss minimiser"}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--config", default="c3_array256")
    ap.add_argument("--cpu-budget", type=float, default=10.0,
                    help="seconds of CPU work for the cpu_baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true", help="skip the host-buffer e2e run")
    ap.add_argument("--no-extras", action="store_true",
                    help="only the headline measurement (profiling runs)")
    ap.add_argument("--sections", default="all",
                    help="comma-separated extra sections to run (accuracy, paths, link, "
                         "station_c2, library_bar, batched, differentiation) or all")
    ap.add_argument("--precision", choices=list(PREC), default="fp16",
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

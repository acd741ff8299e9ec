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

Multi-GPU (torchrun): replicas only -- every rank runs its own 16-integration
stream (different seed), no data-path collective; value = all ranks'
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

# DRAM bytes per launch of the dominant kernels from ncu captures (see
# profiles/fengine_f32_c2.txt and profiles/xengine_f32_c2.txt), scaled to
# the c2 launch; None until a capture exists.
NCU_TRAFFIC = {"fengine_f32": None, "xengine_herm_f32": None}


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

    iq = torch.empty(total_sp * sb, dtype=torch.int8, device=dev)
    ssig, sdel = cfg.sources()
    mdt.synth_iq(cfg.seed + 7919 * rank, ne, nch, 0, total_sp, t(cfg.sigma_q8()), iq,
                 tone_q16=t(cfg.tone_q16()), src_sigma_q8=t(ssig), src_delay=t(sdel))
    win = torch.empty(nch * ntaps, dtype=torch.float32, device=dev)
    mdt.window_hamming_sinc(nch, ntaps, win)
    vis = torch.empty(nint, nch, ne, ne, dtype=torch.complex64, device=dev)
    stream = torch.cuda.current_stream(dev)
    plan = mdt.FxPlan(ne, nch, ntaps, nsp, stream=stream)
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
    kernels = {
        "fengine_f32": {"ms_per_launch": f_launch_ms, "bound": "hbm", "achieved": f_gbs,
                        "unit": "GB/s", "peak": hbm, "frac": f_gbs / hbm,
                        "algorithmic_bytes": f_bytes},
        "xengine_herm_f32": {"ms_per_launch": x_launch_ms, "bound": "fp32", "achieved": x_tflops,
                             "unit": "TFLOP/s", "peak": fp32_peak, "frac": x_tflops / fp32_peak,
                             "algorithmic_flops": x_flops, "hbm_gbs": x_gbs},
    }
    if f_launch_ms >= x_launch_ms:
        name = "fengine_f32"
        roof = {"kernel": name, "bound": "hbm", "achieved": f_gbs, "peak": hbm, "unit": "GB/s",
                "frac": f_gbs / hbm, "traffic": NCU_TRAFFIC[name],
                "peak_source": peak_kind + " hbm_gbs"}
    else:
        name = "xengine_herm_f32"
        roof = {"kernel": name, "bound": "fp32", "achieved": x_tflops, "peak": fp32_peak,
                "unit": "TFLOP/s", "frac": x_tflops / fp32_peak, "traffic": NCU_TRAFFIC[name],
                "peak_source": "nominal FP32 FMA rate (%d SMs x 128 lanes x 2) at the sampled "
                               "SM clock" % nsm}

    # ---- e2e through the host-buffer C-ABI entry (pinned host memory)
    e2e = None
    if not args.no_e2e:
        h_iq = torch.empty(total_sp * sb, dtype=torch.int8, pin_memory=True)
        h_iq.copy_(iq)
        h_vis = torch.empty(nint * nch * ne * ne * 2, dtype=torch.float32, pin_memory=True)
        plan.execute_host(h_iq, nint, h_vis)  # warm-up: staging buffers
        e2e_steps = max(1, min(args.steps, 5))
        barrier()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            plan.execute_host(h_iq, nint, h_vis)
        barrier()
        e2e_s = (time.perf_counter() - t0) / e2e_steps
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
               "api": "mdt_fx_execute_host", "matches_device_run": bool(ok)}

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
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded integer int8 I/Q generator)",
            "config": {"workload": cfg.name, "nelements": ne, "nchannels": nch, "ntaps": ntaps,
                       "nspectra": nsp, "integrations": nint, "path": "fused FP32 plan API",
                       "l2": "inputs (%.1f GB) larger than L2, no flush" % (iq.numel() / 1e9)},
            "e2e": e2e,
            "gpu_launches": 2 * nint * args.steps,
            "roofline": roof,
            "kernels": kernels,
            "cpu_baseline": cpu,
            "clocks": clk,
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
    if args.impl == "reference":
        run_reference(args, cfg)
    else:
        run_ours(args, cfg)


if __name__ == "__main__":
    main()

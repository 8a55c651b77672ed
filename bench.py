#!/usr/bin/env python
"""RK steps/s of the DYNAMITE per-step hot path on GB300.

Workload (the plain FP64 form at L=512): mixed p-spin f(q)=(1-lam)q^3+lam q^4
with lam=0.5 (-p 3 -q 4 -l 0.5), quench from infinite temperature to
Gamma=0.6, poly-9 stencil tables (Tmax=1e5, spline order 5, alpha=delta=0)
generated in-process.  The run starts at t=0, advances `--setup` controller
iterations untimed (history grows to ~setup rows), then times `--steps`
controller iterations (one RK step each, adaptive step size, RK54 /
SSPRK(10,4) as the reference's controller chooses).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Multi-GPU runs are independent replicas (one quench per GPU, no collective).
Prints one JSON line on rank 0.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RK steps/s at L=512 (plain FP64 form)"
UNIT = "steps/s"
L2_BYTES = 129 * 1024 * 1024
STAGEDEV_BYTES = 640     # sizeof(StageDev) per stage, uploaded each step
SLOTS_BYTES = 88         # sizeof(Slots), read back each step


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--setup", type=int, default=1500)
    ap.add_argument("--L", type=int, default=512)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-mixed", dest="mixed", action="store_false", help="skip the mixed-precision measurement")
    return ap.parse_args()


def model_kw():
    return dict(p=3, p2=4, lam=0.5, T0=1e50, Gamma=0.6, delta_t_min=1e-5, delta_max=1e-10)


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class Clocks:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.path = os.path.join(ROOT, "gpurun_out", f"clocks_{device}.csv")

    def __enter__(self):
        os.makedirs(os.path.dirname(self.path), exist_ok=True)
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.device), "-lms", "200"], stdout=self.fh,
                                         stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            self.proc.wait(timeout=5)
            self.fh.close()

    def summary(self):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def read_profile_traffic():
    """DRAM bytes per k_main launch from the committed ncu summary, if any."""
    path = os.path.join(ROOT, "profiles", "k_main_fp64_L512.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def cpu_port_steps_per_s(st_dict, grid, seconds: float, max_steps: int):
    """The C restatement of the reference (oracle/) on the host cores, from the
    same state, until `seconds` of CPU work or `max_steps` steps."""
    import oracle as O
    O.build(reference=False)
    og = O.Grid(grid.L, grid.theta, grid.phi1, grid.phi2, grid.integ, grid.indsA1, grid.wA1, grid.indsA2,
                grid.wA2, grid.indsB2, grid.wB2)
    port = O.Port(og, O.Model(**model_kw()), search_mode=0, threads=0)
    port.set_state(O.State(*st_dict["state"]))
    port.interpolate()
    port.set_controller(st_dict["dt"], st_dict["method"], st_dict["delta"], st_dict["delta_old"], st_dict["loop"])
    t0 = time.perf_counter()
    k = 0
    while k < max_steps and (time.perf_counter() - t0) < seconds:
        port.run(1)
        k += 1
    el = time.perf_counter() - t0
    return k / el, k, el


def run_reference(args):
    """The reference CPU path on the host cores (oracle/_ref where the reference
    compiled here, otherwise the C restatement), same workload."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    import oracle as O
    import dynamite_gb300 as D
    grid = D.grid.generate(args.L)
    og = O.Grid(grid.L, grid.theta, grid.phi1, grid.phi2, grid.integ, grid.indsA1, grid.wA1, grid.indsA2,
                grid.wA2, grid.indsB2, grid.wB2)
    kind, impl = "port", None
    if os.path.exists(O.REF_FAST_LIB):
        try:
            O.Reference.lib(fast=True)
            impl = O.Reference(og, O.Model(**model_kw()), threads=os.cpu_count())
            kind = "reference"
        except OSError:
            impl = None
    if impl is None:
        O.build(reference=False)
        impl = O.Port(og, O.Model(**model_kw()), search_mode=0, threads=0)
    cores = os.cpu_count()
    impl.init_state()
    setup = min(args.setup, 30)
    impl.run(setup)
    for _ in range(min(args.warmup, 3)):
        impl.run(1)
    t0 = time.perf_counter()
    k = 0
    while k < args.steps and (time.perf_counter() - t0) < args.cpu_seconds:
        impl.run(1)
        k += 1
    el = time.perf_counter() - t0
    v = k / el
    out = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": k,
        "warmup": min(args.warmup, 3), "ms_per_step": 1e3 * el / k, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"mixed p-spin lam=0.5 T=0.6 quench, L={args.L}, poly-9 grid, "
                                f"{setup} setup steps from t=0", "L": args.L},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": cores, "kind": kind,
                         "sample": f"{k} controller iterations after {setup} setup steps"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out))


def run_ours(args):
    import torch

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo", init_method="env://")
    from dynamite_gb300 import build as B
    B.build()
    import dynamite_gb300 as D
    from dynamite_gb300.simulation import probe_fp64

    dev = local
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(device=dev)
    grid = D.grid.generate(args.L)
    cap = args.setup + args.warmup + 2 * args.steps + 64
    sim = D.Simulation(grid, D.Model(**model_kw()), device=dev, use_graph=True, history_capacity=cap,
                       stream=stream.cuda_stream)
    sim.init()
    sim.run(args.setup)
    # state for the CPU baseline (same point of the same run)
    cpu_state = None
    if rank == 0 and world == 1:
        st = sim.download()
        c = sim.controller
        cpu_state = {"state": (st.t1grid, st.dtr, st.QK, st.QR, st.dQK, st.dQR, st.rvec, st.drvec),
                     "dt": c["delta_t"], "method": c["method"], "delta": c["delta"], "delta_old": c["delta_old"],
                     "loop": c["loop"]}
    sim.run(args.warmup)
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device=f"cuda:{dev}")

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # ---- device-timed: state resident, L2 flushed before each step (outside the events)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    methods = []
    barrier()
    torch.cuda.synchronize()
    with Clocks(dev) as clk:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            ev[k][0].record(stream)
            out = sim.run(1)
            ev[k][1].record(stream)
            methods.append(int(out["method"][0]))
        torch.cuda.synchronize()
    barrier()
    dev_ms = sum(a.elapsed_time(b) for a, b in ev)
    t_dev = dev_ms / 1e3
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_dev], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_dev = float(tt[0])
    value = world * args.steps / t_dev
    stages = [7 if m == 1 else (10 if m == 2 else 4 * (m - 2)) for m in methods]

    # ---- end to end through the C ABI: host buffers, copies inside the timed region
    qk, qr = np.empty(args.L), np.empty(args.L)
    e2e_steps = max(20, args.steps // 4)
    h2d = d2h = 0
    t_e2e = 0.0
    for k in range(e2e_steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        torch.cuda.synchronize()
        m = sim.controller["method"]
        t0 = time.perf_counter()
        sim.run(1)
        sim.last_row(qk, qr)
        t_e2e += time.perf_counter() - t0
        S = 7 if m == 1 else (10 if m == 2 else 4 * (m - 2))
        h2d += S * STAGEDEV_BYTES
        d2h += SLOTS_BYTES + 2 * args.L * 8
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_e2e], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_e2e = float(tt[0])
    e2e_value = world * e2e_steps / t_e2e

    # ---- the mixed-precision form on the same state (FP32 gathers/convolutions)
    mixed = None
    if args.mixed:
        st0 = sim.download()
        c0 = sim.controller
        msim = D.Simulation(grid, D.Model(**model_kw()), precision="mixed", device=dev, use_graph=True,
                            history_capacity=cap, stream=stream.cuda_stream)
        msim.upload(st0)
        msim.set_controller(c0["delta_t"], c0["method"], c0["delta"], c0["delta_old"], c0["loop"])
        msim.run(args.warmup)
        mev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
        torch.cuda.synchronize()
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            mev[k][0].record(stream)
            msim.run(1)
            mev[k][1].record(stream)
        torch.cuda.synchronize()
        t_mix = sum(a.elapsed_time(b) for a, b in mev) / 1e3
        mm, me = msim.profile_stage(reps=20)
        mixed = {"value": args.steps / t_mix, "unit": UNIT, "ms_per_step": 1e3 * t_mix / args.steps,
                 "stage_ms": {"main": mm, "epilogue": me},
                 "speedup_vs_fp64": (args.steps / t_mix) / (args.steps / (dev_ms / 1e3))}
        msim.close()

    if rank != 0:
        return
    # ---- roofline of the dominant kernel (gather + convolution), timed live
    ms_main, ms_epi = sim.profile_stage(reps=20)
    L, m = args.L, grid.depth
    alg_bytes = 3 * L * L * (8 * m + 4) + 8 * L * L + 8 * L + 16 * L
    alg_flop = (24 * m + 122) * L * L
    peaks, src = measured_peaks()
    fp64_peak = probe_fp64(dev)
    achieved_gbs = alg_bytes / (ms_main * 1e-3) / 1e9
    achieved_fp64 = alg_flop / (ms_main * 1e-3) / 1e9
    traffic = read_profile_traffic()
    cpu = None
    if cpu_state is not None:
        v, k, el = cpu_port_steps_per_s(cpu_state, grid, args.cpu_seconds, args.steps)
        cpu = {"value": v, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
               "sample": f"{k} controller iterations ({el:.1f} s) from the GPU run's state after {args.setup} steps"}
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * t_dev / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"mixed p-spin lam=0.5 T=0.6 quench, L={L}, poly-9 grid (Tmax 1e5), timed after "
                               f"{args.setup} setup steps", "L": L, "history_rows": sim.n,
                   "l2": "flushed before every timed step (256 MB write, outside the events)",
                   "parallelism": "replicas" if world > 1 else "single"},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d / e2e_steps,
                "d2h_bytes_per_step": d2h / e2e_steps},
        "gpu_launches": int(2 * sum(stages)),
        "roofline": {"bound": "hbm", "achieved": achieved_gbs, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved_gbs / peaks["hbm_gbs"], "traffic": traffic,
                     "kernel": "k_main (fused gather+convolution)", "ms_per_launch": ms_main,
                     "peak_source": src},
        "roofline_fp64": {"bound": "fp64", "achieved": achieved_fp64, "peak": fp64_peak, "unit": "GFLOP/s",
                          "frac": achieved_fp64 / fp64_peak, "flop_per_launch": alg_flop,
                          "peak_source": "measured (dyn_probe_fp64, same run)"},
        "stage_ms": {"main": ms_main, "epilogue": ms_epi},
        "clocks": clk.summary(),
        "cpu_baseline": cpu,
        "mixed": mixed,
    }
    print(json.dumps(line))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()

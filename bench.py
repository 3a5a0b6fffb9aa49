#!/usr/bin/env python3
"""Headline benchmark: grid-cell RK3 steps/s of the dry convective boundary
layer LES at 512 x 512 x 256 (Advec_2i5, Smagorinsky with Monin-Obukhov
surface, Boussinesq thermodynamics, Pres_2, RK3, fixed dt = 2 s) in the FP32
form, with the plain FP64 path measured on the same GPU beside it.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

With N > 1 (torchrun, one process per GPU) every rank advances its own
independently seeded member of the same case: the simulation itself has no
data-parallel split on one GPU per member (replicas only), so `value` is the
sum over ranks and `scaling` is "weak".

`--impl reference` times the reference algorithm's CPU implementation (the
oracle port of the reference's hot-path code, OpenMP on all host cores) on the
same case and prints its line; on ranks > 0 it exits without work.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "grid-cell RK3 steps/s"
UNIT = "cell-steps/s"
# Compulsory field passes per RK3 step of the fused pipeline (3 substeps x 52:
# viscosity 5, tendencies 13, pressure rhs 7, FFTs 8, z-solve 2, gradient +
# RK3 update 17); one pass reads or writes one interior field once.
PASSES_PER_STEP = 156
# Passes per launch of each timed kernel group (one substep's worth).
PASSES = {"tendency": 13, "viscosity": 5, "presout_rk3": 17, "pres_in": 7,
          "fft_x": 2, "fft_y": 2, "tdma": 2, "pres_scatter": 2}


def peak_hbm():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(kernel):
    """Per-launch DRAM bytes of kernel group `kernel` at the bench size, from
    the committed ncu summaries (profiles/traffic_*.txt), or None."""
    import glob
    for path in sorted(glob.glob(os.path.join(ROOT, "profiles", "traffic_*.txt"))):
        try:
            for line in open(path):
                if line.startswith("traffic_per_launch_bytes") and f" {kernel} " in line:
                    return float(line.split()[-1])
        except OSError:
            pass
    return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def _allreduce(x, world, op):
    """One float reduced over the ranks (NCCL on the GPUs; gloo on the host
    when the process group is a gloo one, as in the multi-process tests)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=op)
    return float(t.item())


def allreduce_max(x, world):
    import torch.distributed as dist
    return _allreduce(x, world, dist.ReduceOp.MAX)


def allreduce_sum(x, world):
    import torch.distributed as dist
    return _allreduce(x, world, dist.ReduceOp.SUM)


def make_case(size, rank, ktot=None):
    from microhh_gb300 import cases
    n = size
    kt = ktot or n // 2
    return cases.drycbl(n, n, kt, 50. * n, 50. * n, 4000. * kt / (n // 2), seed=2 + rank, name=f"drycbl_{n}x{n}x{kt}")


def bench_config(size, kt, world):
    """The `config` of both arms' lines (the same workload)."""
    return {"workload": f"dry CBL LES {size}x{size}x{kt}, domain {50*size}x{50*size}x{4000. * kt / (size // 2):g} m, "
                        "Advec_2i5 + Smagorinsky (cs 0.23) + MOST surface + Boussinesq + Pres_2, RK3, dt=2 s",
            "parallelism": f"replicas x{world}",
            "l2": "inputs larger than L2 (one field 277 MB), no flush"}


def timed_steps(model, steps, world):
    """Device time of `steps` RK3 steps (CUDA events on the model's stream)."""
    import torch
    barrier(world)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    model.run_steps(steps, fused=True)
    e1.record()
    torch.cuda.synchronize()
    barrier(world)
    return e0.elapsed_time(e1) / 1e3


def cpu_baseline_sample(size, kt, substeps=3):
    """The oracle port of the reference's hot-path code on all host cores:
    `substeps` RK3 substeps of the same case (seconds, cores)."""
    from oracle import orcpy
    orcpy.build()
    case = make_case(size, 0, kt)
    m = orcpy.model_from_case(case)
    cores = m.lib.orc_num_threads()
    t0 = time.perf_counter()
    m.run_substeps(substeps)
    dt = time.perf_counter() - t0
    m.close()
    return dt, cores


def run_reference(args, world, rank):
    """The reference algorithm's CPU implementation on the same case: each
    bench step is one full RK3 step (three substeps) of the whole grid, after
    the warm-up steps; rank 0 alone runs."""
    if rank != 0:
        return
    from oracle import orcpy
    orcpy.build()
    size = args.size
    kt = args.ktot or size // 2
    n = size * size * kt
    case = make_case(size, 0, kt)
    m = orcpy.model_from_case(case)
    cores = m.lib.orc_num_threads()
    m.run_substeps(3 * args.warmup)
    t0 = time.perf_counter()
    m.run_substeps(3 * args.steps)
    total = time.perf_counter() - t0
    m.close()
    value = n * args.steps / total
    sample = (f"{args.steps} RK3 steps of drycbl {size}x{size}x{kt} after {args.warmup} warm-up steps "
              "(oracle port of the reference's hot-path code, FP64, OpenMP on all host cores)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 0,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded dry CBL, theta noise +-0.1 K below 200 m)",
            "config": bench_config(size, kt, world),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args, world, rank, local):
    import numpy as np
    import torch
    import microhh_gb300 as mhh

    size = args.size
    kt = args.ktot or size // 2
    n = size * size * kt
    case = make_case(size, rank, kt)

    # ---- FP32 form: device-resident throughput -------------------------
    m = mhh.Model(case, precision=mhh.FP32)
    m.run_steps(args.warmup, fused=True)
    m.synchronize()
    mhh.Timing.reset()
    mhh.Timing.enable(True)
    clocks = ClockSampler(local)
    clocks.start()
    launches0 = mhh.launch_count()
    secs = timed_steps(m, args.steps, world)
    launches = mhh.launch_count() - launches0
    clk = clocks.stop()
    mhh.Timing.enable(False)
    timing = mhh.Timing.collect()
    secs = allreduce_max(secs, world)
    value = allreduce_sum(n * args.steps / secs, world)
    ms_per_step = 1e3 * secs / args.steps
    cfl, div = m.cfl(), m.div()

    # ---- end to end through the public model API with host buffers -----
    # One job: H2D of the initial state from page-locked host memory, K RK3
    # steps each followed by the status read-back (CFL to the host), D2H of
    # the final state.
    names = case.prognostic_names()
    host_in = {nm: torch.from_numpy(case.embed(case.fields[nm]).astype(np.float32)).pin_memory() for nm in names}
    host_out = {nm: torch.empty_like(host_in[nm]).pin_memory() for nm in names}
    m2 = mhh.Model(case, precision=mhh.FP32)
    m2.run_steps(1, fused=True)
    # Untimed passes over the same page-locked buffers: on the GB300 machine the
    # first two device passes over pinned pages that the CPU has written cost
    # about 10x a later one (13-20 ms against 1.3-1.5 ms per 277 MB field),
    # a one-time cost that a job reusing its staging buffers pays once.
    for _ in range(2):
        for nm in names:
            m2.set_native(nm, host_in[nm].data_ptr())
            m2.get_native(nm, host_out[nm].data_ptr())
        m2.synchronize()
    barrier(world)
    t0 = time.perf_counter()
    for nm in names:
        m2.set_native(nm, host_in[nm].data_ptr())
    for _ in range(args.steps):
        m2.run_steps(1, fused=True)
        m2.cfl()
    for nm in names:
        m2.get_native(nm, host_out[nm].data_ptr())
    m2.synchronize()
    e2e_secs = allreduce_max(time.perf_counter() - t0, world)
    bytes_state = sum(t.numel() * t.element_size() for t in host_in.values())
    e2e = {"value": allreduce_sum(n * args.steps / e2e_secs, world), "unit": UNIT,
           "h2d_bytes_per_step": bytes_state / args.steps,
           "d2h_bytes_per_step": bytes_state / args.steps + 8,
           "job": f"H2D state, {args.steps} RK3 steps with a CFL read-back each, D2H state"}
    del m2
    del m
    torch.cuda.synchronize()

    # ---- plain FP64 path on the same GPU --------------------------------
    fp64 = None
    if args.fp64_steps > 0:
        m64 = mhh.Model(case, precision=mhh.FP64)
        m64.run_steps(1, fused=True)
        s64 = allreduce_max(timed_steps(m64, args.fp64_steps, world), world)
        v64 = allreduce_sum(n * args.fp64_steps / s64, world)
        fp64 = {"value": v64, "unit": UNIT, "ms_per_step": 1e3 * s64 / args.fp64_steps,
                "steps": args.fp64_steps, "fp32_over_fp64": value / v64,
                "note": "plain FP64 path, same case and kernels' FP64 builds, device-resident"}
        del m64

    # ---- roofline of the dominant kernel --------------------------------
    peak, peak_kind = peak_hbm()
    groups = {k: v for k, v in timing.items() if k in PASSES}
    dom = max(groups, key=lambda k: groups[k][1]) if groups else None
    roof = None
    if dom:
        cnt, ms = groups[dom]
        bytes_launch = PASSES[dom] * n * 4
        achieved = bytes_launch / (ms / cnt / 1e3) / 1e9
        roof = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": bytes_launch,
                "traffic": ncu_traffic(dom), "avg_launch_ms": ms / cnt}
    step_bytes = PASSES_PER_STEP * n * 4
    step_roof = {"achieved": step_bytes / (secs / args.steps) / 1e9, "peak": peak, "unit": "GB/s",
                 "frac": step_bytes / (secs / args.steps) / 1e9 / peak}
    kernels = {k: {"launch_groups": v[0], "total_ms": round(v[1], 3), "ms_per_step": round(v[1] / args.steps, 3)}
               for k, v in sorted(timing.items(), key=lambda kv: -kv[1][1])}

    # ---- CPU baseline (rank 0, N = 1) ----------------------------------
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        dt, cores = cpu_baseline_sample(size, kt, 3)
        cpu = {"value": n / dt, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": f"1 RK3 step of drycbl {size}x{size}x{kt} (oracle port of the reference's hot-path code, "
                         "FP64, OpenMP)"}
        if fp64:
            # Like for like: the FP64 GPU path against the FP64 CPU code.
            cpu["fp64_gpu_over_cpu"] = fp64["value"] / cpu["value"]
            cpu["fp32_gpu_over_cpu"] = value / cpu["value"]

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32 (FP64 z-solve and reductions)",
                "data": "synthetic (seeded dry CBL, theta noise +-0.1 K below 200 m)",
                "config": bench_config(size, kt, world),
                "fp64": fp64, "e2e": e2e, "roofline": roof, "step_roofline": step_roof,
                "cpu_baseline": cpu, "clocks": clk, "gpu_launches": launches, "kernels": kernels,
                "diagnostics": {"cfl": cfl, "div": div}}
        print(json.dumps(line), flush=True)


def run_form(args):
    """The batching (64-member ensemble) and serving forms on one GPU."""
    # Many concurrent streams: let each map to its own hardware queue (the
    # default of 8 would serialise streams that share one).  Read when the
    # CUDA context is created, so it is set before the first CUDA call.
    os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")
    import microhh_gb300 as mhh
    from microhh_gb300 import forms
    if args.form == "ensemble":
        r = forms.ensemble_workload(mhh)
        line = {"metric": "ensemble member-cell RK3 steps/s", "value": max(r["graphs"], r["batched"]), "unit": "cell-steps/s",
                "n_gpus": 1, "higher_is_better": True, "form": "ensemble", "dtype": "f32 (FP64 z-solve)",
                "data": "synthetic (seeded dry CBL members)", "config": {"workload": r["workload"]},
                "detail": r}
    else:
        r = forms.serve_workload(mhh)
        line = {"metric": "served cell RK3 steps/s", "value": r["saturated"]["continuous"]["throughput"],
                "unit": "cell-steps/s", "n_gpus": 1, "higher_is_better": True, "form": "serve",
                "dtype": "f32 (FP64 z-solve)", "data": "synthetic (seeded dry CBL jobs)",
                "config": {"workload": r["workload"]}, "detail": r}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--ktot", type=int, default=0, help="vertical levels (default size/2)")
    ap.add_argument("--fp64-steps", type=int, default=10)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--form", default="step", choices=["step", "ensemble", "serve"],
                    help="step: the time-step throughput (default); ensemble / serve: the batching and "
                         "serving forms, one JSON line each")
    args = ap.parse_args()
    if args.form != "step":
        run_form(args)
        return
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        world = int(os.environ.get("WORLD_SIZE", "1"))
        run_reference(args, world, rank)
        return
    world, rank, local = dist_setup()
    run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

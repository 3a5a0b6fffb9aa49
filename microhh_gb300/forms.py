"""The batching and serving forms of the time step, as measured workloads.

ensemble_workload: 64 dry-CBL members with grids drawn from {32^3, 48x48x64,
64^3, 96x96x64, 128x128x96}, surface heat flux ~ U[0.05, 0.25] K m/s and lapse
rate ~ U[0.001, 0.006] K/m, each with its own seed (member m: seed 3 + m), FP32
form, dt = 2 s.  Timed one member after another and as one CUDA-graph launch
per RK3 substep after autotuning.

serve_workload: jobs with cubic grids n ~ log-uniform[32, 256] quantised to
2^a 3^b 5^c, dry CBL physics with sbot ~ U[0.05, 0.25], FP32 form, a device
memory budget of 150 GB.  The step counts are drawn from [50, 300] (the full
workload asks for 100-2000; the range is scaled so that one run takes seconds).
Measured saturated (all jobs at t = 0, throughput of the serving loop against
the same jobs one after another) and under Poisson arrivals at 80% of the
serving loop's saturated job rate (p50 and p99 latency in both modes).
"""
import math
import time

import numpy as np

from . import cases

ENSEMBLE_GRIDS = [(32, 32, 32), (48, 48, 64), (64, 64, 64), (96, 96, 64), (128, 128, 96)]


def ensemble_cases(nmembers=64, seed=3):
    rng = np.random.default_rng(seed)
    out = []
    for m in range(nmembers):
        itot, jtot, ktot = ENSEMBLE_GRIDS[int(rng.integers(len(ENSEMBLE_GRIDS)))]
        sbot = float(rng.uniform(0.05, 0.25))
        lapse = float(rng.uniform(0.001, 0.006))
        out.append(cases.drycbl(itot, jtot, ktot, 100. * itot, 100. * jtot, 4000., seed=3 + m, sbot=sbot,
                                lapse=lapse, noise_z=400., name=f"member{m}_{itot}x{jtot}x{ktot}"))
    return out


def smooth_sizes(lo=32, hi=256):
    vals = set()
    for a in range(0, 9):
        for b in range(0, 6):
            for c in range(0, 4):
                n = 2**a * 3**b * 5**c
                if lo <= n <= hi and n % 2 == 0:
                    vals.add(n)
    return sorted(vals)


def serve_cases(njobs, seed=4, steps=(50, 300)):
    rng = np.random.default_rng(seed)
    sizes = np.array(smooth_sizes())
    out = []
    for j in range(njobs):
        target = math.exp(rng.uniform(math.log(32), math.log(256)))
        n = int(sizes[np.argmin(np.abs(np.log(sizes) - math.log(target)))])
        sbot = float(rng.uniform(0.05, 0.25))
        nsteps = int(rng.integers(steps[0], steps[1] + 1))
        c = cases.drycbl(n, n, n, 50. * n, 50. * n, 4000., seed=4 + j, sbot=sbot, noise_z=400.,
                         name=f"job{j}_{n}")
        out.append((c, nsteps))
    return out


def ensemble_workload(mhh, nmembers=64, steps=5):
    import torch
    cs = ensemble_cases(nmembers)
    models = [mhh.Model(c, precision=mhh.FP32) for c in cs]
    cells = sum(c.itot * c.jtot * c.ktot for c in cs)
    ens = mhh.Ensemble(models)

    def timed(mode, n):
        ens.synchronize()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ens.run_steps(n, mode)
        ens.synchronize()
        return time.perf_counter() - t0

    timed(mhh.ENS_SEQUENTIAL, 1)
    t_seq = timed(mhh.ENS_SEQUENTIAL, steps)
    report = ens.autotune()
    timed(mhh.ENS_GRAPHS, 2)          # eager step + capture
    n0 = mhh.launch_count()
    t_graph = timed(mhh.ENS_GRAPHS, steps)
    launches = mhh.launch_count() - n0
    timed(mhh.ENS_BATCHED, 2)         # eager step + batch plan + capture
    n0 = mhh.launch_count()
    t_batch = timed(mhh.ENS_BATCHED, steps)
    launches_b = mhh.launch_count() - n0
    timed(mhh.ENS_STREAMS, 1)
    t_streams = timed(mhh.ENS_STREAMS, steps)
    ens.close()
    for m in models:
        m.close()
    return {
        "workload": f"{nmembers} dry-CBL members, grids from {ENSEMBLE_GRIDS}, FP32 form",
        "member_cells": cells,
        "steps": steps,
        "sequential": cells * steps / t_seq,
        "streams": cells * steps / t_streams,
        "graphs": cells * steps / t_graph,
        "batched": cells * steps / t_batch,
        "graphs_over_sequential": t_seq / t_graph,
        "batched_over_sequential": t_seq / t_batch,
        "graph_kernel_launches_per_step": launches / steps,
        "batched_kernel_launches_per_step": launches_b / steps,
        "autotune": report,
    }


def serve_workload(mhh, njobs=48, budget=150e9, max_active=16):
    jobs = serve_cases(njobs)
    total = sum(c.itot * c.jtot * c.ktot * n for c, n in jobs)

    def run(mode, arrivals):
        srv = mhh.Server(budget, max_active)
        ids = [srv.submit(c, n, arrival=a) for (c, n), a in zip(jobs, arrivals)]
        t0 = time.perf_counter()
        srv.run(mode)
        wall = time.perf_counter() - t0
        times = [srv.times(j) for j in ids]
        peak = srv.peak_bytes()
        t, c = srv.progress()
        srv.close()
        lat = np.array([f - a for a, _, f in times])
        makespan = max(f for _, _, f in times) - min(a for a, _, _ in times)
        # Sustained rate: cells stepped between 10% and 90% of the total work,
        # over the time that took (excludes the ramp-up and the tail of the
        # finite job list).
        order = np.argsort(t, kind="stable")
        cum = np.cumsum(c[order])
        tt = t[order]
        i10 = int(np.searchsorted(cum, 0.1 * cum[-1]))
        i90 = int(np.searchsorted(cum, 0.9 * cum[-1]))
        sustained = (cum[i90] - cum[i10]) / max(tt[i90] - tt[i10], 1e-9)
        return {"throughput": total / makespan, "sustained": float(sustained),
                "p50_s": float(np.percentile(lat, 50)),
                "p99_s": float(np.percentile(lat, 99)), "makespan_s": makespan, "wall_s": wall,
                "peak_budget_bytes": peak}

    zero = [0.0] * njobs
    sat_cont = run(mhh.SERVE_CONTINUOUS, zero)
    sat_fifo = run(mhh.SERVE_FIFO, zero)
    # Poisson arrivals at 80% of the serving loop's saturated job rate.
    rate = 0.8 * njobs / sat_cont["makespan_s"]
    rng = np.random.default_rng(44)
    arr = np.cumsum(rng.exponential(1.0 / rate, njobs))
    arr -= arr[0]
    poi_cont = run(mhh.SERVE_CONTINUOUS, list(arr))
    poi_fifo = run(mhh.SERVE_FIFO, list(arr))
    return {
        "workload": f"{njobs} dry-CBL jobs, cubic n log-uniform in [32, 256] (2^a3^b5^c), 50-300 steps, FP32 form",
        "cell_steps": total,
        "budget_bytes": budget, "max_active": max_active,
        "saturated": {"continuous": sat_cont, "fifo": sat_fifo,
                      "continuous_over_fifo": sat_cont["throughput"] / sat_fifo["throughput"],
                      "sustained_continuous_over_fifo": sat_cont["sustained"] / sat_fifo["sustained"]},
        "poisson": {"rate_jobs_per_s": rate, "continuous": poi_cont, "fifo": poi_fifo},
    }

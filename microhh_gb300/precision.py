"""Precision study of the FP32 form against the plain FP64 path.

cbl_study: the large dry CBL (512x512x256, 25600x25600x4000 m, seeded theta
noise of +-0.1 K below 200 m, dt = 2 s) run for `steps` steps in both
precisions; the horizontal mean and variance profiles of u, v, w and theta are
averaged over the last `avg` steps (300 steps = 10 minutes).

channel_study: the turbulent channel DNS (256x192x128, Re_tau ~ 180,
adaptive dt) for `steps` steps; mean-velocity and RMS profiles averaged over
the last `avg` steps.

Errors are reported per quantity, normalised by the FP64 profile's own scale:
the maximum over the interior levels of |f32 - f64| divided by the maximum of
|f64| (means of w, u, v: by the square root of the maximum FP64 variance, as
their means are near zero; theta mean: by the range of the FP64 profile).
"""
import time

import numpy as np

from . import cases


def _averaged(mhh, case, precision, steps, avg, names):
    m = mhh.Model(case, precision=precision)
    g = m.grid
    t0 = time.perf_counter()
    m.run_steps(steps - avg)
    acc = {n: [np.zeros(g.kcells), np.zeros(g.kcells)] for n in names}
    for _ in range(avg):
        m.run_steps(1)
        for n in names:
            mean, var = m.profile_stats(n)
            acc[n][0] += mean / avg
            acc[n][1] += var / avg
    m.synchronize()
    secs = time.perf_counter() - t0
    ks = slice(g.kstart, g.kend)
    out = {n: (acc[n][0][ks], acc[n][1][ks]) for n in names}
    m.close()
    return out, secs


def _compare(p32, p64):
    res = {}
    for n in p64:
        m32, v32 = p32[n]
        m64, v64 = p64[n]
        vscale = max(np.abs(v64).max(), 1e-300)
        if n == "th":
            mscale = max(m64.max() - m64.min(), 1e-300)
        elif n in ("u", "v", "w") and np.abs(m64).max() < np.sqrt(vscale):
            mscale = np.sqrt(vscale)
        else:
            mscale = max(np.abs(m64).max(), 1e-300)
        res[n] = {"mean_err": float(np.abs(m32 - m64).max() / mscale),
                  "var_err": float(np.abs(v32 - v64).max() / vscale),
                  "mean_scale": float(mscale), "var_scale": float(vscale)}
    return res


def cbl_study(mhh, size=512, steps=1800, avg=300):
    case = cases.drycbl(size, size, size // 2, 50. * size, 50. * size, 4000., seed=2)
    names = ("u", "v", "w", "th")
    p32, s32 = _averaged(mhh, case, mhh.FP32, steps, avg, names)
    p64, s64 = _averaged(mhh, case, mhh.FP64, steps, avg, names)
    return {"case": f"dry CBL {size}x{size}x{size//2}, dt=2 s, {steps} steps, profiles averaged over the last {avg}",
            "errors": _compare(p32, p64), "seconds_fp32": s32, "seconds_fp64": s64,
            "profiles_fp64": {n: [p64[n][0].tolist(), p64[n][1].tolist()] for n in names},
            "profiles_fp32": {n: [p32[n][0].tolist(), p32[n][1].tolist()] for n in names}}


def channel_study(mhh, steps=2000, avg=500):
    case = cases.channel(256, 192, 128, seed=1)
    names = ("u", "v", "w")
    p32, s32 = _averaged(mhh, case, mhh.FP32, steps, avg, names)
    p64, s64 = _averaged(mhh, case, mhh.FP64, steps, avg, names)
    return {"case": f"channel DNS 256x192x128 Re_tau~180, adaptive dt, {steps} steps, profiles averaged over the last {avg}",
            "errors": _compare(p32, p64), "seconds_fp32": s32, "seconds_fp64": s64}


def cbl_fp64_floor(mhh, size=512, steps=1800, avg=300):
    """The same FP64 run with the tridiagonal solve in the rescaled
    recurrence (a change of round-off only, 1e-16 per operation): its
    difference from the plain FP64 run is the chaotic-divergence floor that
    any FP32-vs-FP64 comparison of these statistics sits on."""
    case = cases.drycbl(size, size, size // 2, 50. * size, 50. * size, 4000., seed=2)
    names = ("u", "v", "w", "th")
    mhh.set_option("tdma_kernel", 1)
    try:
        p, secs = _averaged(mhh, case, mhh.FP64, steps, avg, names)
    finally:
        mhh.set_option("tdma_kernel", -1)
    return {"case": f"dry CBL {size}x{size}x{size//2}, FP64 with the rescaled tridiagonal recurrence",
            "seconds_fp64": secs, "profiles_fp64_perturbed": {n: [p[n][0].tolist(), p[n][1].tolist()] for n in names}}


def cbl_fp64_float_start(mhh, size=512, steps=1800, avg=300):
    """The FP64 path started from the float-rounded initial state (theta
    rounded to float, as the FP32 form stores it): its difference from the
    plain FP64 run is how far the flow alone carries an initial perturbation
    of float size, the yardstick for the FP32 form's differences."""
    case = cases.drycbl(size, size, size // 2, 50. * size, 50. * size, 4000., seed=2)
    case.fields["th"] = case.fields["th"].astype(np.float32).astype(np.float64)
    names = ("u", "v", "w", "th")
    p, secs = _averaged(mhh, case, mhh.FP64, steps, avg, names)
    return {"case": f"dry CBL {size}x{size}x{size//2}, FP64 from the float-rounded initial theta",
            "seconds_fp64": secs, "profiles_fp64_floatstart": {n: [p[n][0].tolist(), p[n][1].tolist()] for n in names}}


if __name__ == "__main__":
    import argparse
    import json
    import microhh_gb300 as mhh
    ap = argparse.ArgumentParser()
    ap.add_argument("--which", default="both", choices=["cbl", "channel", "both", "floor", "floatstart"])
    ap.add_argument("--size", type=int, default=512)
    ap.add_argument("--steps", type=int, default=1800)
    ap.add_argument("--avg", type=int, default=300)
    a = ap.parse_args()
    out = {}
    if a.which == "floatstart":
        print(json.dumps({"floatstart": cbl_fp64_float_start(mhh, a.size, a.steps, a.avg)}), flush=True)
    if a.which == "floor":
        print(json.dumps({"floor": cbl_fp64_floor(mhh, a.size, a.steps, a.avg)}), flush=True)
    if a.which in ("channel", "both"):
        out["channel"] = channel_study(mhh)
        print(json.dumps({"channel": out["channel"]}), flush=True)
    if a.which in ("cbl", "both"):
        out["cbl"] = cbl_study(mhh, a.size, a.steps, a.avg)
        print(json.dumps({"cbl": out["cbl"]}), flush=True)

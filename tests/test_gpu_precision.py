"""The precision form against the FP64 oracle over a 10-minute average.

The dry CBL at 64x64x64 (6400x6400x4000 m, dt = 2 s) runs 600 steps
in the oracle, the plain FP64 path and the FP32 form; the horizontal mean and
variance profiles of u, v, w and theta are averaged over the last 300 steps
(10 minutes) and compared level by level with the oracle's, normalised as in
microhh_gb300.precision (means of u, v, w by the velocity scale sqrt(max var),
theta's mean by its range, variances by their maximum).

Bounds:
- FP64: round-off only.  The fields end 1.6e-11 (relative L2) from the
  oracle's and the averaged profiles 3e-13; held to 1e-9 and 1e-10.
- FP32 form: 0.5% for every averaged profile (measured
  2.4e-6 on a GB300); the fields themselves are held to 1e-2 relative L2
  (measured 1.4e-4 for u).
"""
import numpy as np
import pytest

from microhh_gb300 import cases, precision

pytestmark = pytest.mark.gpu

STEPS, AVG = 600, 300
NAMES = ("u", "v", "w", "th")


@pytest.fixture(scope="module")
def mhh():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import microhh_gb300
    microhh_gb300.load()
    return microhh_gb300


@pytest.fixture(scope="module")
def oracle_run(oracle_lib):
    """The oracle's averaged profiles and final fields."""
    case = cases.drycbl()
    o = oracle_lib.model_from_case(case)
    ks = slice(case.kgc, case.kgc + case.ktot)
    g = case.igc
    o.run_substeps(3 * (STEPS - AVG))
    acc = {n: [np.zeros(case.ktot), np.zeros(case.ktot)] for n in NAMES}
    for _ in range(AVG):
        o.run_substeps(3)
        for n in NAMES:
            a = o.get(n)[ks, g:g + case.jtot, g:g + case.itot]
            mean = a.mean(axis=(1, 2))
            acc[n][0] += mean / AVG
            acc[n][1] += ((a - mean[:, None, None]) ** 2).mean(axis=(1, 2)) / AVG
    fields = {n: o.get(n) for n in NAMES}
    o.close()
    return case, {n: (acc[n][0], acc[n][1]) for n in NAMES}, fields


@pytest.mark.parametrize("prec,tol_prof,tol_field", [(64, 1e-10, 1e-9), (32, 5e-3, 1e-2)], ids=["fp64", "fp32"])
def test_averaged_profiles_against_oracle(mhh, oracle_run, prec, tol_prof, tol_field):
    case, po, fo = oracle_run
    p, _ = precision._averaged(mhh, case, prec, STEPS, AVG, NAMES)
    errs = precision._compare(p, po)
    for n in NAMES:
        assert errs[n]["mean_err"] <= tol_prof, (n, errs[n])
        assert errs[n]["var_err"] <= tol_prof, (n, errs[n])
    m = mhh.Model(case, precision=prec)
    m.run_steps(STEPS)
    for n in NAMES:
        ref = fo[n] - (case.thref0 if n == "th" else 0.)
        err = float(np.linalg.norm(m.get(n) - fo[n]) / np.linalg.norm(ref))
        assert err <= tol_field, (n, err)
    m.close()

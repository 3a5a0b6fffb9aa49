"""Failure detection on the device path: non-finite fields are reported.

The failures are made on the host: a NaN (or an out-of-range velocity) is
written into a field through the public model API, and the tests expect the
reductions to return MHH_ERR_NONFINITE and the time loop's status check
(src/model.cxx:842-872) to stop the run with "Simulation has non-finite
numbers".  No kernel faults, traps or waits.
"""
import ctypes

import numpy as np
import pytest

from microhh_gb300 import cases

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mhh():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import microhh_gb300
    microhh_gb300.load()
    return microhh_gb300


def small_case():
    return cases.drycbl(32, 24, 16, 3200., 2400., 1600., seed=81, noise_z=400.)


def with_value(m, case, name, value, cell=(5, 7, 9)):
    a = m.get(name)
    kg = case.kgc
    g = 3 if case.advec == "2i5" else 1
    a[cell[0] + kg, cell[1] + g, cell[2] + g] = value
    m.set(name, a)


@pytest.mark.parametrize("precision", [64, 32], ids=["fp64", "fp32"])
def test_reductions_report_nan(mhh, precision):
    """One NaN in u makes the CFL and divergence maxima NaN (fmax would drop
    it); one NaN in evisc makes the diffusion number NaN."""
    case = small_case()
    m = mhh.Model(case, precision=precision)
    m.run_steps(1)
    assert np.isfinite(m.cfl()) and np.isfinite(m.div()) and np.isfinite(m.dn())
    with_value(m, case, "u", np.nan)
    for what in (m.cfl, m.div):
        with pytest.raises(mhh.MhhError) as e:
            what()
        assert e.value.status == mhh.ERR_NONFINITE, what
    m2 = mhh.Model(case, precision=precision)
    m2.run_steps(1)
    with_value(m2, case, "evisc", np.nan)
    with pytest.raises(mhh.MhhError) as e:
        m2.dn()
    assert e.value.status == mhh.ERR_NONFINITE
    m.close(); m2.close()


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "modules"])
def test_status_check_stops_a_blown_up_run(mhh, fused):
    """The status check at the start of a step (iteration % outputiter == 0)
    stops the run on a NaN velocity, as the reference's print_status does."""
    case = small_case()
    m = mhh.Model(case, precision=mhh.FP64)
    m.run_steps(1, fused=fused)
    with_value(m, case, "w", np.nan)
    # outputiter defaults to 20: iteration 1 is not checked, so the NaN
    # spreads until iteration 20, where the check stops the run.  The
    # module-by-module loop computes the time-step limits at every step, and
    # their CFL reduction already reports the NaN.
    with pytest.raises(mhh.MhhError, match="non-finite|not finite") as e:
        m.run_steps(25, fused=fused)
    assert e.value.status == mhh.ERR_NONFINITE
    m.close()


def test_status_check_cfl_out_of_range(mhh):
    """A finite but huge velocity (CFL >= 10) also stops the run at the
    first checked iteration, as in the reference (!(cfl >= 0 && cfl < 10))."""
    case = small_case()
    m = mhh.Model(case, precision=mhh.FP64)
    with_value(m, case, "u", 1.e5)
    with pytest.raises(mhh.MhhError, match="non-finite") as e:
        m.run_steps(1)
    assert e.value.status == mhh.ERR_NONFINITE
    m.close()


def test_healthy_run_passes_checks(mhh):
    """outputiter = 0 checks every substep; a healthy run is not stopped."""
    case = small_case()
    ini = case.to_ini().replace("[time]", "[time]\noutputiter=0")
    m = mhh.Model(ini=ini, z=case.z, precision=mhh.FP64)
    for n in case.prognostic_names():
        m.set(n, case.embed(case.fields[n]))
    m.run_steps(3)
    assert np.isfinite(m.cfl())
    m.close()

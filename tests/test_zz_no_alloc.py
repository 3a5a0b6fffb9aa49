"""mhh_pres_2_get_divergence_noalloc against mhh_pres_2_get_divergence.

Both are called through the C-ABI on the same device fields, twice in a row
on different states, in FP64 and FP32 contexts.  The two compute the same
per-cell expression and take exact maxima, so they agree to the FP64
tolerance of the parity tests (1e-12 relative, or 1e-12 of the divergence
scale where the divergence is at round-off after a projection).
"""
import ctypes

import numpy as np
import pytest

from microhh_gb300 import cases

pytestmark = pytest.mark.gpu

TOL = 1e-12


@pytest.fixture(scope="module")
def mhh():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import microhh_gb300
    kern, _ = microhh_gb300.load()
    f = kern.mhh_pres_2_get_divergence_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.POINTER(microhh_gb300.Fields), ctypes.POINTER(ctypes.c_double),
                  ctypes.c_void_p]
    return microhh_gb300


def both(mhh, m):
    kern, _ = mhh.load()
    fl, _ = m.device_fields()
    a, b = ctypes.c_double(), ctypes.c_double()
    mhh.check(kern.mhh_pres_2_get_divergence(m.ctx(), ctypes.byref(fl), ctypes.byref(a), None), "divergence")
    mhh.check(kern.mhh_pres_2_get_divergence_noalloc(m.ctx(), ctypes.byref(fl), ctypes.byref(b), None),
              "divergence_noalloc")
    return a.value, b.value


def scale(case, m):
    dzi = 1.0 / np.diff(np.concatenate([[0.0], 0.5 * (case.z[1:] + case.z[:-1]), [case.zsize]]))
    return (np.abs(m.get("u")).max() * case.itot / case.xsize + np.abs(m.get("v")).max() * case.jtot / case.ysize
            + np.abs(m.get("w")).max() * dzi.max())


@pytest.mark.parametrize("precision", [64, 32], ids=["fp64", "fp32"])
def test_noalloc_divergence_matches(mhh, precision):
    case = cases.drycbl(32, 24, 16, 3200., 2400., 1600., seed=41, noise_z=400.)
    m = mhh.Model(case, precision=precision)
    rng = np.random.default_rng(7)
    shape = m.get("u").shape
    # Two calls in a row on two non-solenoidal states.
    for call in range(2):
        for n in ("u", "v", "w"):
            a = rng.standard_normal(shape)
            if precision == 32:
                a = a.astype(np.float32).astype(np.float64)
            m.set(n, a)
        ref, got = both(mhh, m)
        assert ref > 0
        assert abs(got - ref) <= TOL * ref, (call, got, ref)
    # And after a projection, where the divergence is at round-off.
    m.run_steps(1)
    ref, got = both(mhh, m)
    assert abs(got - ref) <= TOL * scale(case, m), (got, ref)


def test_noalloc_divergence_at_the_size_limit(mhh):
    """jtot*ktot = 262144 row maxima exactly (the largest accepted use of
    the scratch array, with the row index spanning the whole grid of
    blocks), two calls in a row, against mhh_pres_2_get_divergence."""
    case = cases.drycbl(8, 512, 512, 800., 51200., 5120., seed=43, noise_z=200.)
    m = mhh.Model(case, precision=mhh.FP64)
    rng = np.random.default_rng(8)
    shape = m.get("u").shape
    for call in range(2):
        for n in ("u", "v", "w"):
            m.set(n, rng.standard_normal(shape))
        ref, got = both(mhh, m)
        assert ref > 0
        assert abs(got - ref) <= TOL * ref, (call, got, ref)
    m.close()


@pytest.mark.parametrize("precision", [64, 32], ids=["fp64", "fp32"])
def test_noalloc_divergence_reports_nan(mhh, precision):
    """One NaN in u gives MHH_ERR_NONFINITE from both divergence entry
    points (a maximum that dropped the NaN would report a finite value)."""
    kern, _ = mhh.load()
    case = cases.drycbl(32, 24, 16, 3200., 2400., 1600., seed=44, noise_z=400.)
    m = mhh.Model(case, precision=precision)
    u = m.get("u")
    u[5, 10, 11] = np.nan
    m.set("u", u)
    fl, _ = m.device_fields()
    out = ctypes.c_double()
    assert kern.mhh_pres_2_get_divergence(m.ctx(), ctypes.byref(fl), ctypes.byref(out), None) == mhh.ERR_NONFINITE
    assert kern.mhh_pres_2_get_divergence_noalloc(m.ctx(), ctypes.byref(fl), ctypes.byref(out), None) == mhh.ERR_NONFINITE
    assert np.isnan(out.value)
    m.close()


def test_noalloc_divergence_rejects_large_grid(mhh):
    """jtot*ktot above the 262144 row maxima of the scratch array is an
    argument error (no launch, no allocation)."""
    kern, _ = mhh.load()
    case = cases.drycbl(8, 1080, 256, 800., 108000., 4000., seed=42, noise_z=200.)
    m = mhh.Model(case, precision=32)
    fl, _ = m.device_fields()
    out = ctypes.c_double()
    rc = kern.mhh_pres_2_get_divergence_noalloc(m.ctx(), ctypes.byref(fl), ctypes.byref(out), None)
    assert rc == -1
    assert b"262144" in kern.mhh_last_error()

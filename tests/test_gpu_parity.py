"""CUDA path against the oracle and the reference's golden fixtures.

All calls go through the C-ABI (libmhh_gb300.so) and the host layer
(libmhh_host.so).  FP64: 1e-12 relative per field after one RK3 step (the
parity requirement of the FP64 path against the reference's FP64 CPU build).  FP32 form: compared with the
FP64 oracle at the tolerance stated per test.
"""
import glob
import os

import numpy as np
import pytest

from microhh_gb300 import cases

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
TOL64 = 1e-12
# The eddy viscosity is mlen^2 |S| sqrt(1 - N2/(S2 Pr)) with the ratio clipped
# at 1 - 1e-9 (src/diff_smag2.cxx:171-174): where the ratio approaches the clip,
# a 1e-16 change of N2 or S2 changes evisc by up to 1e-16/(1 - ratio), so this
# diagnostic field is held to 1e-9 while the prognostic fields and p are held
# to 1e-12.
TOL_EVISC = 1e-9


def rel_err(a, b):
    """Norm-wise relative error ||a - b||_2 / ||b||_2."""
    scale = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / (scale if scale > 0 else 1.0))


def read_levels(case, name, a):
    """The levels of a field that the time step reads.  With two vertical
    ghost levels (flux-limited Advec_2i5) the reference's Pres_2 uses the
    storage of p as scratch for the packed transform and never rewrites
    level kstart-2, which no module reads (src/pres_2.cxx:155-196, 330-358):
    that level is left out of comparisons of p."""
    if name == "p" and case.kgc == 2:
        return a[case.kgc - 1:]
    return a


def max_err(a, b):
    """Largest pointwise error relative to the field's largest magnitude."""
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / (scale if scale > 0 else 1.0))


@pytest.fixture(scope="module")
def mhh():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import microhh_gb300
    microhh_gb300.load()
    return microhh_gb300


def golden_case(name):
    from tests.golden.make_golden import golden_cases
    return golden_cases()[name]


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "modules"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_golden_fp64(mhh, path, fused):
    name = os.path.basename(path)[:-4]
    g = np.load(path)
    case = golden_case(name)
    m = mhh.Model(case, precision=mhh.FP64)
    for n in case.prognostic_names():
        m.set(n, g["in_" + n])
    for key in g.files:
        if key.startswith("buf_"):
            m.set_buffer_profile(key[4:], g[key])
    m.run_substeps(3, fused=fused)
    for key in g.files:
        if key.startswith("out_"):
            n = key[4:]
            err = rel_err(read_levels(case, n, m.get(n)), read_levels(case, n, g[key]))
            assert err <= (TOL_EVISC if n == "evisc" else TOL64), (name, n, err)
    assert m.dt() == float(g["diag_dt"])
    for d in ("cfl", "dn"):
        ref = float(g["diag_" + d])
        got = getattr(m, d)()
        assert abs(got - ref) <= TOL64 * abs(ref), (name, d, got, ref)
    from tests.test_oracle import div_scale
    assert m.div() <= TOL64 * div_scale(case, g), (name, m.div())


LARGER = [
    ("cbl_64x48x32", lambda: cases.drycbl(64, 48, 32, 6400., 4800., 3200., seed=21, noise_z=800.)),
    ("cbl_60x40x24_radix35", lambda: cases.drycbl(60, 40, 24, 6000., 4000., 2400., seed=22, noise_z=600.)),
    ("channel_48x36x32", lambda: cases.channel(48, 36, 32, seed=23, dt=5e-4, adaptivestep=True)),
]


# The larger cases are held to the same 1e-12 for one RK3 step.  Both the
# oracle and the CUDA path evaluate the inverse transforms with each level's
# mean mode set aside and added back at the end, so the strong hydrostatic
# part of the pressure does not put order-dependent round-off into the
# horizontal pressure gradient (without that, two valid CPU FFTs differing
# only in the order of their radix passes differed by 1.4e-12 in u after one
# step of cbl_64x48x32; with it, by 1.7e-13).  What remains is the rounding
# of p = p' + mean itself, which the two paths share except where their p'
# differ across a rounding boundary.  Two steps are held to TOL_LARGE2.
TOL_LARGE = 1e-12
TOL_LARGE2 = 2e-12


@pytest.mark.parametrize("name,make", LARGER, ids=[n for n, _ in LARGER])
def test_against_oracle_fp64(mhh, oracle_lib, name, make):
    case = make()
    m = mhh.Model(case, precision=mhh.FP64)
    o = oracle_lib.model_from_case(case)
    for nsteps, tol in ((1, TOL_LARGE), (2, TOL_LARGE2)):
        m.run_steps(nsteps, fused=True)
        o.run_substeps(3 * nsteps)
        for n in case.prognostic_names() + ["p"]:
            a, b = m.get(n), o.get(n)
            err = rel_err(a, b)
            assert err <= tol, (name, n, nsteps, err)
            assert max_err(a, b) <= 10 * tol, (name, n, nsteps, max_err(a, b))


def test_drycbl_64cubed_fp64_1_and_100_steps(mhh, oracle_lib):
    """The dry CBL configuration exactly (64x64x64, 6400x6400x4000 m,
    Advec_2i5, Smagorinsky, Monin-Obukhov surface, dt = 2 s): one RK3 step at
    the FP64 tolerance, then 100 steps at TOL_100.

    Over 100 steps round-off differences grow with the flow: two valid CPU
    FFTs that differ only in the order of their radix passes end 1.6e-11 (u,
    v) and 2.0e-11 (w) apart after 100 steps of this case, so the CUDA path is
    held to five times that."""
    TOL_100 = 1e-10
    case = cases.drycbl()
    assert (case.itot, case.jtot, case.ktot, case.zsize, case.dt) == (64, 64, 64, 4000., 2.)
    m = mhh.Model(case, precision=mhh.FP64)
    o = oracle_lib.model_from_case(case)
    done = 0
    for nsteps, tol in ((1, TOL_LARGE), (100, TOL_100)):
        m.run_steps(nsteps - done, fused=True)
        o.run_substeps(3 * (nsteps - done))
        done = nsteps
        for n in case.prognostic_names() + ["p"]:
            err = rel_err(m.get(n), o.get(n))
            assert err <= tol, (n, nsteps, err)
    assert abs(m.cfl() - o.cfl()) <= TOL_100 * o.cfl()
    m.close(); o.close()


def test_channel_256x192x128_fp64(mhh, oracle_lib):
    """The channel DNS configuration exactly (256x192x128, tanh-stretched
    wall-normal levels, Advec_2, Diff_2, dpdx forcing, adaptive time step):
    one RK3 step at the FP64 tolerance."""
    case = cases.channel()
    assert (case.itot, case.jtot, case.ktot) == (256, 192, 128)
    m = mhh.Model(case, precision=mhh.FP64)
    o = oracle_lib.model_from_case(case)
    m.run_steps(1, fused=True)
    o.run_substeps(3)
    assert m.dt() == o.dt()
    for n in case.prognostic_names() + ["p"]:
        err = rel_err(m.get(n), o.get(n))
        assert err <= TOL_LARGE, (n, err)
    m.close(); o.close()


# Channel in the FP32 form against the FP64 oracle from the same
# float-representable state: the velocities (~15 u_tau) are stored to half a
# float ulp per update, a relative 3e-8, and the float FFTs and stencils add
# errors of the same order per substep (measured on a GB300: at most 5e-7
# relative for w after one step); one step is held to TOL_CH32.
TOL_CH32 = 5e-6


@pytest.mark.parametrize("name,make", [
    ("channel_48x36x32", lambda: cases.channel(48, 36, 32, seed=23, dt=5e-4, adaptivestep=True)),
    ("channel_256x192x128", lambda: cases.channel()),
], ids=["channel_48x36x32", "channel_256x192x128"])
def test_channel_fp32_form_against_fp64_oracle(mhh, oracle_lib, name, make):
    case = make()
    for n in case.fields:
        case.fields[n] = case.fields[n].astype(np.float32).astype(np.float64)
    m = mhh.Model(case, precision=mhh.FP32)
    o = oracle_lib.model_from_case(case)
    m.run_steps(1, fused=True)
    o.run_substeps(3)
    for n in case.prognostic_names():
        err = rel_err(m.get(n), o.get(n))
        assert err <= TOL_CH32, (name, n, err)
    m.close(); o.close()


@pytest.mark.parametrize("variant", [0, 1, 2], ids=["percell", "tiled", "flux"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_tendency_variants_fp64(mhh, path, variant):
    """Every LES tendency kernel (per cell in the reference's operation order;
    tiled planes; flux form, the default) on double fields against the golden
    fixtures at the FP64 tolerance."""
    name = os.path.basename(path)[:-4]
    g = np.load(path)
    case = golden_case(name)
    mhh.set_option("tendency_kernel", variant)
    try:
        m = mhh.Model(case, precision=mhh.FP64)
        for n in case.prognostic_names():
            m.set(n, g["in_" + n])
        m.run_substeps(3, fused=True)
        for n in case.prognostic_names() + ["p"]:
            err = rel_err(read_levels(case, n, m.get(n)), read_levels(case, n, g["out_" + n]))
            assert err <= TOL64, (name, n, err)
    finally:
        mhh.set_option("tendency_kernel", -1)


@pytest.mark.parametrize("variant", [0, 1], ids=["percell", "planes"])
@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_viscosity_planes_fp64(mhh, path, variant):
    """Both eddy-viscosity kernels (per cell; plane-staged, the default) on
    double fields against the golden fixtures (evisc at its own tolerance,
    the rest at FP64)."""
    name = os.path.basename(path)[:-4]
    g = np.load(path)
    case = golden_case(name)
    mhh.set_option("viscosity_kernel", variant)
    try:
        m = mhh.Model(case, precision=mhh.FP64)
        for n in case.prognostic_names():
            m.set(n, g["in_" + n])
        m.run_substeps(3, fused=True)
        for key in g.files:
            if key.startswith("out_"):
                n = key[4:]
                err = rel_err(read_levels(case, n, m.get(n)), read_levels(case, n, g[key]))
                assert err <= (TOL_EVISC if n == "evisc" else TOL64), (name, n, err)
    finally:
        mhh.set_option("viscosity_kernel", -1)


@pytest.mark.parametrize("variant", [0, 2], ids=["percell", "flux"])
def test_tendency_chunks_and_partial_tiles_fp64(mhh, oracle_lib, variant):
    """A grid whose x and y sizes are not multiples of the tile and whose
    height spans three level chunks (the last one partial), against the
    oracle."""
    case = cases.drycbl(40, 20, 70, 4000., 2000., 2800., seed=24, noise_z=600.)
    mhh.set_option("tendency_kernel", variant)
    mhh.set_option("viscosity_kernel", 1 if variant == 2 else 0)
    try:
        m = mhh.Model(case, precision=mhh.FP64)
        o = oracle_lib.model_from_case(case)
        m.run_steps(1, fused=True)
        o.run_substeps(3)
        for n in case.prognostic_names() + ["p"]:
            err = rel_err(m.get(n), o.get(n))
            assert err <= TOL_LARGE, (n, err)
    finally:
        mhh.set_option("tendency_kernel", -1)
        mhh.set_option("viscosity_kernel", -1)


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_tdma_rescaled_recurrence_fp64(mhh, path):
    """The rescaled Thomas recurrence of the float form (two FP64 FMAs per
    cell), run on double fields, against the golden fixtures at the FP64
    tolerance."""
    name = os.path.basename(path)[:-4]
    g = np.load(path)
    case = golden_case(name)
    mhh.set_option("tdma_kernel", 1)
    try:
        m = mhh.Model(case, precision=mhh.FP64)
        for n in case.prognostic_names():
            m.set(n, g["in_" + n])
        m.run_substeps(3, fused=True)
        for n in case.prognostic_names() + ["p"]:
            err = rel_err(read_levels(case, n, m.get(n)), read_levels(case, n, g["out_" + n]))
            assert err <= TOL64, (name, n, err)
    finally:
        mhh.set_option("tdma_kernel", -1)


@pytest.mark.parametrize("xsize", [6400., 320000.], ids=["float_groups", "mixed_groups"])
def test_tdma_float_groups_match_fp64_elimination(mhh, xsize):
    """The float form's default solve (float sweeps for the column groups
    whose forward sweep damps, FP64 for the rest) against the same step with
    every group eliminated in FP64: norm-wise relative differences of 2e-6
    in the pressure and 1e-6 in the velocities.  At 320 km (5 km spacing over 15.6 m
    levels) the lowest horizontal modes keep FP64; at 6.4 km every group but
    the mean mode runs in float."""
    case = cases.drycbl(64, 64, 64, xsize, xsize, 1000., seed=33, noise_z=400.)
    out = {}
    for v in (1, 3):
        mhh.set_option("tdma_kernel", v)
        try:
            m = mhh.Model(case, precision=mhh.FP32)
            m.run_substeps(1, fused=True)
            out[v] = {n: m.get(n) for n in ("p", "u", "v", "w")}
            m.close()
        finally:
            mhh.set_option("tdma_kernel", -1)
    for n, tol in (("p", 2e-6), ("u", 1e-6), ("v", 1e-6), ("w", 1e-6)):
        err = rel_err(out[3][n], out[1][n])
        assert err <= tol, (n, err)


@pytest.mark.parametrize("variant", [0, 2], ids=["percell", "flux"])
def test_fp32_form_against_fp64_oracle(mhh, oracle_lib, variant):
    """FP32 storage/stencils/FFTs with FP64 z-solve and reductions: one RK3
    step within 2e-3 of the FP64 oracle (relative to each field's maximum).

    The bound is set by storage: theta ~ 300 K in float carries an absolute
    error of 1.5e-5 K, i.e. 1.5e-4 of the 0.1 K noise that drives the flow."""
    case = cases.drycbl(64, 48, 32, 6400., 4800., 3200., seed=31, noise_z=800.)
    # Start both from the same float-representable state.
    case.fields["th"] = case.fields["th"].astype(np.float32).astype(np.float64)
    mhh.set_option("tendency_kernel", variant)
    try:
        m = mhh.Model(case, precision=mhh.FP32)
        m.run_steps(1, fused=True)
    finally:
        mhh.set_option("tendency_kernel", -1)
    o = oracle_lib.model_from_case(case)
    o.run_substeps(3)
    for n in ("u", "v", "w"):
        err = rel_err(m.get(n), o.get(n))
        assert err <= 2e-3, (n, err)
    # Potential temperature (~300 K) is stored to half an ulp, 1.5e-5 K, per
    # update: three RK3 substeps stay within 1e-4 K of the FP64 oracle.
    assert np.abs(case.interior(m.get("th") - o.get("th"))).max() <= 1e-4


@pytest.mark.parametrize("itot,jtot", [(48, 40), (42, 56), (50, 36), (70, 30)])
def test_fft_roundtrip_and_dft(mhh, itot, jtot):
    """Forward transforms against numpy's DFT in halfcomplex order, and the
    inverse pair returns itot*jtot times the input (fixed and run-time-plan
    lengths with the radices 2, 3, 4, 5, 7, 8)."""
    import ctypes
    import torch
    ktot = 3
    desc = mhh.GridDesc(itot, jtot, ktot, 1, 1, 1, 1.0, 1.0, 1.0)
    phys = mhh.Physics(visc=1e-5, svisc=1e-5, cs=0.23, tpr=1/3., dnmax=0.4, swmason=1, cflmax=1.,
                       thref0=300., thermo=0, surface=0, z0m=0.1, z0h=0.1)
    z = np.linspace(0.1, 0.9, ktot)
    h = ctypes.c_void_p()
    kern, _ = mhh.load()
    mhh.check(kern.mhh_ctx_create(ctypes.byref(desc), z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  64, ctypes.byref(phys), ctypes.byref(h)))
    rng = np.random.default_rng(3)
    x = rng.standard_normal((ktot, jtot, itot))
    t = torch.tensor(x, dtype=torch.float64, device="cuda")
    mhh.check(kern.mhh_fft_forward(h, ctypes.c_void_p(t.data_ptr()), None))
    torch.cuda.synchronize()
    got = t.cpu().numpy()
    X = np.fft.fft2(x, axes=(1, 2))   # complex (ky, kx)
    # Halfcomplex along x then along y: build the expected array.
    def hc(a, axis):
        n = a.shape[axis]
        F = np.fft.fft(a, axis=axis)
        out = np.empty(a.shape)
        idx = [slice(None)] * a.ndim
        for k in range(n // 2 + 1):
            idx[axis] = k
            out[tuple(idx)] = F[tuple(idx)].real
        for k in range(1, (n + 1) // 2):
            idx[axis] = n - k
            src = list(idx); src[axis] = k
            out[tuple(idx)] = F[tuple(src)].imag
        return out
    exp = hc(hc(x, 2), 1)
    assert np.abs(got - exp).max() <= 1e-12 * np.abs(exp).max()
    mhh.check(kern.mhh_fft_backward(h, ctypes.c_void_p(t.data_ptr()), None))
    torch.cuda.synchronize()
    back = t.cpu().numpy()
    assert np.abs(back - itot * jtot * x).max() <= 1e-12 * itot * jtot * np.abs(x).max()
    kern.mhh_ctx_destroy(h)
    del X


@pytest.mark.parametrize("pipe", [1, 0], ids=["prefetching", "tile_per_block"])
@pytest.mark.parametrize("precision", [64, 32], ids=["fp64", "fp32"])
@pytest.mark.parametrize("n", [128, 256, 512])
def test_fft_warp_schedule(mhh, n, precision, pipe):
    """The warp-synchronous schedule (n = 64 R, R = 2, 4, 8; rows and columns,
    both FFT kernels) against numpy's DFT in halfcomplex order, and the
    inverse pair returning itot*jtot times the input."""
    import ctypes
    import torch
    itot = jtot = n
    ktot = 3
    desc = mhh.GridDesc(itot, jtot, ktot, 1, 1, 1, 1.0, 1.0, 1.0)
    phys = mhh.Physics(visc=1e-5, svisc=1e-5, cs=0.23, tpr=1/3., dnmax=0.4, swmason=1, cflmax=1.,
                       thref0=300., thermo=0, surface=0, z0m=0.1, z0h=0.1)
    z = np.linspace(0.1, 0.9, ktot)
    h = ctypes.c_void_p()
    kern, _ = mhh.load()
    mhh.check(kern.mhh_ctx_create(ctypes.byref(desc), z.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                  precision, ctypes.byref(phys), ctypes.byref(h)))
    rng = np.random.default_rng(5)
    x = rng.standard_normal((ktot, jtot, itot))
    dt = torch.float64 if precision == 64 else torch.float32
    # Float: the transforms' round-off, a few eps times log2(n).
    tol = 1e-12 if precision == 64 else 3e-6
    mhh.set_option("fft_pipeline", pipe)
    try:
        t = torch.tensor(x, dtype=dt, device="cuda")
        mhh.check(kern.mhh_fft_forward(h, ctypes.c_void_p(t.data_ptr()), None))
        torch.cuda.synchronize()
        got = t.double().cpu().numpy()
        # Halfcomplex along x, then along y of those rows.
        ref = x if precision == 64 else x.astype(np.float32).astype(np.float64)
        Fx = np.fft.fft(ref, axis=2)
        hx = np.empty_like(x)
        hx[:, :, :itot // 2 + 1] = Fx[:, :, :itot // 2 + 1].real
        hx[:, :, itot // 2 + 1:] = Fx[:, :, 1:itot // 2][:, :, ::-1].imag
        Fy = np.fft.fft(hx, axis=1)
        exp = np.empty_like(x)
        exp[:, :jtot // 2 + 1, :] = Fy[:, :jtot // 2 + 1, :].real
        exp[:, jtot // 2 + 1:, :] = Fy[:, 1:jtot // 2, :][:, ::-1, :].imag
        assert np.abs(got - exp).max() <= tol * np.abs(exp).max()
        mhh.check(kern.mhh_fft_backward(h, ctypes.c_void_p(t.data_ptr()), None))
        torch.cuda.synchronize()
        back = t.double().cpu().numpy()
        assert np.abs(back - itot * jtot * ref).max() <= tol * itot * jtot * np.abs(ref).max()
    finally:
        mhh.set_option("fft_pipeline", 1)
        kern.mhh_ctx_destroy(h)


def test_divergence_after_projection(mhh):
    case = cases.drycbl(48, 32, 24, 4800., 3200., 2400., seed=41, noise_z=800.)
    # FP32: the FFTs and the gradient run in float (eps 6e-8 times the
    # transform length's log and the cancellation of the divergence).
    for prec, tol in ((mhh.FP64, 1e-12), (mhh.FP32, 1e-3)):
        m = mhh.Model(case, precision=prec)
        m.run_steps(2)
        w = np.abs(case.interior(m.get("w"))).max()
        dz = case.zsize / case.ktot
        assert m.div() <= tol * max(w / dz, 1e-30), (prec, m.div(), w / dz)


def test_launches_counted(mhh):
    case = cases.drycbl(32, 24, 16, 3200., 2400., 1600., seed=5)
    m = mhh.Model(case)
    n0 = mhh.launch_count()
    m.run_steps(1)
    assert mhh.launch_count() - n0 >= 3 * 10


@pytest.mark.parametrize("precision", [64, 32], ids=["fp64", "fp32"])
def test_profile_statistics(mhh, precision):
    """Mean and variance profiles on the device against numpy over the
    interior of every level."""
    case = cases.drycbl(40, 24, 20, 4000., 2400., 2000., seed=61, noise_z=600.)
    m = mhh.Model(case, precision=precision)
    m.run_steps(1)
    g = m.grid
    for name in ("u", "w", "th"):
        mean, var = m.profile_stats(name)
        a = m.get(name)[:, g.jstart:g.jend, g.istart:g.iend]
        ref_mean = a.mean(axis=(1, 2))
        ref_var = ((a - ref_mean[:, None, None])**2).mean(axis=(1, 2))
        # Sums of many terms of both signs: round-off relative to the field's
        # magnitude, not to the (possibly near-zero) mean.
        assert np.allclose(mean, ref_mean, rtol=1e-12, atol=1e-13 * np.abs(a).max()), name
        assert np.allclose(var, ref_var, rtol=1e-9, atol=1e-14 * max(ref_var.max(), 1e-30)), name


def test_native_fields_carry_the_scalar_offset(mhh):
    """Native-precision copies of the FP32 form: get_native returns the stored
    anomaly plus thref0 rounded in float (added on the device), set_native
    stores the value minus thref0 rounded in float; the velocities copy as
    they are."""
    case = cases.drycbl(32, 32, 32, 3200., 3200., 3200., seed=71, noise_z=800.)
    m = mhh.Model(case, precision=mhh.FP32)
    m.run_steps(2)
    off = m.scalar_offset()
    assert off == 300.
    for name, o in (("u", 0.), ("th", off)):
        stored = (m.get(name) - o).astype(np.float32)    # exact: float values plus 300 in double
        expect = stored + np.float32(o)
        out = np.empty(m.shape, dtype=np.float32)
        m.get_native(name, out.ctypes.data)
        m.synchronize()
        assert np.array_equal(out, expect), name
        back = (expect * np.float32(1.001)).astype(np.float32)
        m.set_native(name, back.ctypes.data)
        m.synchronize()
        assert np.array_equal((m.get(name) - o).astype(np.float32), back - np.float32(o)), name
    m.close()


@pytest.mark.parametrize("precision", [64, 32], ids=["fp64", "fp32"])
def test_restart_is_bitwise(mhh, precision, tmp_path):
    """Save after two steps, load into a fresh model and run two more: the
    fields equal those of four uninterrupted steps bit for bit (the restart
    test of the reference, python/microhh_tools.py:493-539)."""
    case = cases.drycbl(40, 24, 20, 4000., 2400., 2000., seed=62, noise_z=600.)
    a = mhh.Model(case, precision=precision)
    a.run_steps(4)
    b = mhh.Model(case, precision=precision)
    b.run_steps(2)
    iotime = b.save(str(tmp_path))
    assert iotime == 4
    tf = 8 if precision == 64 else 4
    assert (tmp_path / "th.0000004").stat().st_size == 40 * 24 * 20 * tf
    assert (tmp_path / "time.0000004").stat().st_size == 8 + 8 + 4
    with pytest.raises(mhh.MhhError):
        b.save(str(tmp_path))       # never overwrites
    c = mhh.Model(case, precision=precision)
    c.load(str(tmp_path), iotime)
    c.run_steps(2)
    assert c.time() == a.time()
    for n in case.prognostic_names():
        assert np.array_equal(c.get(n), a.get(n)), n


@pytest.mark.parametrize("precision", [64, 32], ids=["fp64", "fp32"])
def test_pressure_fusion_is_bitwise(mhh, precision):
    """The right-hand side and the scatter fused into the x transforms give
    the same fields bit for bit as the separate kernels (a fixed FFT length
    and a run-time-plan length)."""
    for case in (cases.drycbl(40, 24, 20, 4000., 2400., 2000., seed=63, noise_z=600.),
                 cases.drycbl(60, 40, 24, 6000., 4000., 2400., seed=64, noise_z=600.),
                 cases.drycbl(512, 512, 6, 25600., 25600., 600., seed=67, noise_z=400.)):
        out = []
        for fuse in (0, 1):
            mhh.set_option("pres_fuse", fuse)
            try:
                m = mhh.Model(case, precision=precision)
                m.run_steps(2)
                out.append({n: m.get(n) for n in case.prognostic_names() + ["p"]})
            finally:
                mhh.set_option("pres_fuse", 1)
        for n in out[0]:
            assert np.array_equal(out[0][n], out[1][n]), (case.name, n)


@pytest.mark.parametrize("precision", [64, 32], ids=["fp64", "fp32"])
def test_fft_pipeline_is_bitwise(mhh, precision):
    """The persistent, prefetching FFT kernels give the same fields bit for
    bit as one tile per block (fixed lengths 64, 48, 128, 96, and 512 with
    the warp-synchronous schedule; partial last tiles)."""
    for case in (cases.drycbl(64, 48, 20, 6400., 4800., 2000., seed=65, noise_z=600.),
                 cases.drycbl(128, 96, 13, 12800., 9600., 1300., seed=66, noise_z=600.),
                 cases.drycbl(512, 512, 6, 25600., 25600., 600., seed=68, noise_z=400.)):
        out = []
        for pipe, pairs in ((0, 4), (1, 4), (1, 8)):
            mhh.set_option("fft_pipeline", pipe)
            mhh.set_option("fft_column_pairs", pairs)
            try:
                m = mhh.Model(case, precision=precision)
                m.run_steps(2)
                out.append({n: m.get(n) for n in case.prognostic_names() + ["p"]})
            finally:
                mhh.set_option("fft_pipeline", 1)
                mhh.set_option("fft_column_pairs", 8)
        for q in (1, 2):
            for n in out[0]:
                assert np.array_equal(out[0][n], out[q][n]), (case.name, n, q)


def buffered_cbl(itot, jtot, ktot, seed):
    """A dry CBL with a mean wind and perturbations at every level, and a
    buffer layer (src/buffer.cxx) over the top third of the domain."""
    case = cases.drycbl(itot, jtot, ktot, 100. * itot, 100. * jtot, 100. * ktot, seed=seed, noise_z=100. * ktot)
    rng = np.random.default_rng(seed)
    sh = (ktot, jtot, itot)
    case.fields["u"] = 2. + 0.01 * np.arange(ktot)[:, None, None] + rng.normal(0., 0.3, sh)
    case.fields["v"] = -1. + rng.normal(0., 0.3, sh)
    case.fields["w"] = rng.normal(0., 0.1, sh)
    case.fields["w"][0] = 0.
    case.swbuffer = True
    case.buffer_zstart = 2. / 3. * case.zsize
    case.buffer_sigma = 0.01
    case.buffer_beta = 2.
    return case


@pytest.mark.parametrize("fused", [True, False], ids=["fused", "modules"])
def test_buffer_layer_fp64(mhh, oracle_lib, fused):
    case = buffered_cbl(48, 40, 30, seed=61)
    m = mhh.Model(case, precision=mhh.FP64)
    o = oracle_lib.model_from_case(case)
    m.run_steps(1, fused=fused)
    o.run_substeps(3)
    for n in case.prognostic_names() + ["p"]:
        err = rel_err(m.get(n), o.get(n))
        assert err <= TOL_LARGE, (n, err)
    # The layer acts: without it the upper levels end elsewhere.
    case.swbuffer = False
    off = mhh.Model(case, precision=mhh.FP64)
    off.run_steps(1, fused=fused)
    ktop = case.ktot
    for n in ("u", "v", "w", "th"):
        d = np.abs(off.get(n)[ktop] - m.get(n)[ktop]).max()
        assert d > 1e-6, (n, d)
    m.close(); off.close(); o.close()


def solenoidal_float_start(case, oracle_lib):
    """Replaces the case's initial fields by the oracle's state after one RK3
    step (projected, so divergence-free to FP64 round-off), rounded to float.

    The FP32 form advects theta as its anomaly about thref0 and leaves out
    the term thref0 * div(u) that the flux form of the full theta carries: it
    is zero for the velocity the pressure solve leaves behind, while a float
    divergence residual times 300 K would be as large as the physical
    tendency.  Comparisons of the FP32 form therefore start from a projected
    state, as every step of a run does."""
    o = oracle_lib.model_from_case(case)
    o.run_substeps(3)
    for n in case.prognostic_names():
        case.fields[n] = case.interior(o.get(n)).astype(np.float32).astype(np.float64)
    o.close()
    return case


def test_buffer_layer_fp32(mhh, oracle_lib):
    """FP32 form with the buffer layer against the FP64 oracle, from the same
    float-representable projected state, at the FP32 form's tolerances (2e-3
    relative for the velocities, 1e-4 K per RK3 step for theta)."""
    case = solenoidal_float_start(buffered_cbl(48, 40, 30, seed=62), oracle_lib)
    m = mhh.Model(case, precision=mhh.FP32)
    o = oracle_lib.model_from_case(case)
    m.run_steps(2)
    o.run_substeps(6)
    for n in ("u", "v", "w"):
        err = rel_err(m.get(n), o.get(n))
        assert err <= 2e-3, (n, err)
    assert np.abs(case.interior(m.get("th") - o.get("th"))).max() <= 2e-4
    m.close(); o.close()


def test_buffer_needs_profiles(mhh):
    case = buffered_cbl(16, 16, 12, seed=63)
    m = mhh.Model(ini=case.to_ini(), z=case.z, precision=mhh.FP64)
    with pytest.raises(mhh.MhhError, match="buffer"):
        m.run_steps(1)
    m.close()


def limited_cbl(itot, jtot, ktot, seed):
    """A dry CBL with th advected by the flux limiter ([advec]
    fluxlimit_list=th), a mean wind and a theta front so that the limiter
    clips."""
    case = cases.drycbl(itot, jtot, ktot, 100. * itot, 100. * jtot, 100. * ktot, seed=seed,
                        noise_z=100. * ktot, noise=0.5)
    rng = np.random.default_rng(seed)
    sh = (ktot, jtot, itot)
    case.fields["u"] = 2. + rng.normal(0., 0.5, sh)
    case.fields["v"] = -1. + rng.normal(0., 0.5, sh)
    case.fields["w"] = rng.normal(0., 0.3, sh)
    case.fields["w"][0] = 0.
    case.fields["th"][:, :, itot // 2:] += 1.
    case.fluxlimit = True
    return case


@pytest.mark.parametrize("variant", [0, 2], ids=["percell", "flux"])
def test_flux_limiter_fp64(mhh, oracle_lib, variant):
    """Limited scalar advection on a grid with partial tiles in x and y and
    three level chunks (the last partial), in both tendency kernels, against
    the oracle; the two vertical ghost levels of the limited grid included."""
    case = limited_cbl(40, 20, 70, seed=71)
    mhh.set_option("tendency_kernel", variant)
    mhh.set_option("tendency_kchunk", 32)
    try:
        m = mhh.Model(case, precision=mhh.FP64)
        assert m.grid.kgc == 2
        o = oracle_lib.model_from_case(case)
        m.run_steps(1, fused=True)
        o.run_substeps(3)
        for n in case.prognostic_names() + ["p"]:
            err = rel_err(read_levels(case, n, m.get(n)), read_levels(case, n, o.get(n)))
            assert err <= TOL_LARGE, (n, err)
    finally:
        mhh.set_option("tendency_kernel", -1)
        mhh.set_option("tendency_kchunk", 0)


def test_flux_limiter_fp32(mhh, oracle_lib):
    """FP32 form (flux-form kernel with the limiter) against the FP64 oracle
    from the same float-representable projected state, at the FP32
    tolerances."""
    case = solenoidal_float_start(limited_cbl(48, 40, 30, seed=72), oracle_lib)
    m = mhh.Model(case, precision=mhh.FP32)
    o = oracle_lib.model_from_case(case)
    m.run_steps(1)
    o.run_substeps(3)
    for n in ("u", "v", "w"):
        err = rel_err(m.get(n), o.get(n))
        assert err <= 2e-3, (n, err)
    assert np.abs(case.interior(m.get("th") - o.get("th"))).max() <= 1e-4
    m.close(); o.close()


@pytest.mark.parametrize("precision", [64, 32], ids=["fp64", "fp32"])
def test_flux_limiter_keeps_bounds(mhh, precision):
    """The limiter is monotone: for a two-valued theta field in a uniform
    wind along x, one forward step with the advection tendency of
    mhh_advec_2i5_exec creates no new extrema (CFL 0.1-0.5), where the
    unlimited 5th-order scheme over- and undershoots."""
    import ctypes

    def tendency(limit):
        case = cases.drycbl(32, 8, 8, 3200., 800., 800., seed=73, noise=0.)
        case.fields["u"] = np.full((8, 8, 32), 5.)
        th = np.full((8, 8, 32), 300.)
        th[:, :, 8:16] = 301.
        case.fields["th"] = th
        case.fluxlimit = limit
        m = mhh.Model(case, precision=precision)
        m.set("tht", np.zeros(m.shape))
        f, _ = m.device_fields()
        ctx = m.ctx()
        for p in (f.u, f.v, f.w, f.s):
            mhh.check(m.kern.mhh_boundary_cyclic(ctx, p, 3, None))
        mhh.check(m.kern.mhh_advec_2i5_exec(ctx, ctypes.byref(f), None))
        m.synchronize()
        out = case.interior(m.get("th")), case.interior(m.get("tht"))
        m.close()
        return out
    tol = 1e-12 if precision == 64 else 1e-4
    th, st = tendency(True)
    for dt in (2., 5., 10.):
        new = th + dt * st
        assert new.min() >= 300. - tol and new.max() <= 301. + tol, (dt, new.min(), new.max())
    th, st = tendency(False)
    new = th + 5. * st
    assert new.min() < 300. - 0.1 and new.max() > 301. + 0.1


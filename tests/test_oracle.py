"""The CPU oracle against the reference's own numbers.

The golden fixtures in tests/golden were produced by the reference's hot-path
sources compiled unchanged (tests/golden/make_golden.py); the restatement in
oracle/ must reproduce them after one RK3 step to 1e-12 relative per field.
"""
import glob
import os

import numpy as np
import pytest

from microhh_gb300 import cases

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
TOL = 1e-12


def rel_err(a, b):
    scale = np.abs(b).max()
    return np.abs(a - b).max() / (scale if scale > 0 else 1.0)


def div_scale(case, g):
    """Velocity-gradient scale max|u|/min(dx, dy, dz) of a fixture's output."""
    vmax = max(np.abs(g["out_" + n]).max() for n in ("u", "v", "w"))
    z = case.z
    dz = np.diff(np.concatenate(([0.], 0.5 * (z[1:] + z[:-1]), [case.zsize]))).min()
    return vmax / min(case.xsize / case.itot, case.ysize / case.jtot, dz)


def golden_case(name):
    from tests.golden.make_golden import golden_cases
    return golden_cases()[name]


@pytest.mark.parametrize("path", GOLDEN, ids=[os.path.basename(p)[:-4] for p in GOLDEN])
def test_restatement_matches_reference(oracle_lib, path):
    name = os.path.basename(path)[:-4]
    g = np.load(path)
    case = golden_case(name)
    m = oracle_lib.Model(oracle_lib.params_from_case(case), case.z)
    for n in case.prognostic_names():
        m.set(n, g["in_" + n])
    for key in g.files:
        if key.startswith("buf_"):
            m.set_buffer_profile(key[4:], g[key])
    m.run_substeps(3)
    for key in g.files:
        if key.startswith("out_"):
            n = key[4:]
            err = rel_err(m.get(n), g[key])
            assert err <= TOL, (name, n, err)
    m.lib.orc_set_cyclic_and_ghost(m.h)
    for d in ("cfl", "dn"):
        ref = float(g["diag_" + d])
        got = getattr(m, d)()
        assert abs(got - ref) <= TOL * abs(ref), (name, d, got, ref)
    # After the projection the divergence is round-off: both must be below
    # 1e-12 of the velocity-gradient scale.
    assert max(m.div(), float(g["diag_div"])) <= TOL * div_scale(case, g), name
    assert m.dt() == float(g["diag_dt"])


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 6, 8, 12, 15, 16, 18, 20, 24, 30, 32, 48, 64, 96, 100, 128, 192, 256])
def test_fft_matches_dft(oracle_lib, n):
    """R2HC / HC2R against a direct long-double-free O(n^2) DFT."""
    rng = np.random.default_rng(n)
    x = rng.standard_normal((3, n))
    X = np.fft.fft(x, axis=-1)
    hc = np.empty_like(x)
    for k in range(n // 2 + 1):
        hc[:, k] = X[:, k].real
    for k in range(1, (n + 1) // 2):
        hc[:, n - k] = X[:, k].imag
    got = oracle_lib.r2hc(x)
    assert np.abs(got - hc).max() <= 1e-13 * max(1.0, np.abs(hc).max())
    back = oracle_lib.hc2r(got)
    assert np.abs(back - n * x).max() <= 1e-13 * n * max(1.0, np.abs(x).max())


def test_divergence_free_after_projection(oracle_lib):
    """After a pressure solve the discrete divergence of (u + dt ut) vanishes."""
    case = cases.drycbl(16, 12, 10, 1600., 1200., 1000., seed=5)
    m = oracle_lib.model_from_case(case)
    m.run_substeps(6)
    # The status check runs after the periodic fill of the next substep
    # (src/model.cxx:367-382), so the ghost cells are refreshed first.
    m.lib.orc_set_cyclic_and_ghost(m.h)
    assert m.div() < 1e-12 * max(1.0, np.abs(m.get("w")).max())


def buffered_cbl(itot=24, jtot=20, ktot=16, seed=31):
    """A dry CBL with a mean wind and perturbations at every level, and a
    buffer layer over the top third of the domain."""
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


def test_buffer_restatement(oracle_lib):
    """orc_exec_buffer against src/buffer.cxx:37-59 written out with numpy:
    at -= sigma ((z - zstart)/(zsize - zstart))^beta (a - abuf) at the levels
    with z >= zstart (half levels and abuf = 0 for w)."""
    case = buffered_cbl()
    m = oracle_lib.model_from_case(case)
    fields = {n: case.embed(case.fields[n]) for n in ("u", "v", "w", "th")}
    for n in ("ut", "vt", "wt", "tht"):
        m.set(n, np.zeros(m.shape))
    m.lib.orc_exec_buffer(m.h)
    z = np.zeros(m.kcells)
    z[1:-1] = case.z
    zh = np.zeros(m.kcells)
    zh[2:-1] = 0.5 * (case.z[1:] + case.z[:-1])
    prof = case.buffer_profiles()
    zs, zsize = case.buffer_zstart, case.zsize
    for n, t, lev in (("u", "ut", z), ("v", "vt", z), ("w", "wt", zh), ("th", "tht", z)):
        want = np.zeros(m.shape)
        abuf = prof.get(n, np.zeros(m.kcells))
        for k in range(1, m.kcells - 1):
            if lev[k] < zs:
                continue
            sig = case.buffer_sigma * ((lev[k] - zs) / (zsize - zs)) ** case.buffer_beta
            want[k] = -sig * (fields[n][k] - abuf[k])
        got = m.get(t)
        inner = (slice(1, -1), slice(m.jgc, -m.jgc), slice(m.igc, -m.igc))
        assert np.abs(got[inner] - want[inner]).max() <= 1e-15 * max(1., np.abs(want).max()), n
        assert np.abs(want).max() > 0., n
    m.close()

"""Index algebra of the warp-synchronous FFT schedule and the error bound of
the float tridiagonal sweeps, restated in numpy (CPU).

The GPU kernels (mhh_pres.cu: fft_warp, warp_pos, warp_twiddles, warp_res;
k_tdma_table and tdma_mixed_body) are checked on the device by
tests/test_gpu_parity.py; these tests pin the decomposition and the
precision criterion they are built on.
"""
import numpy as np
import pytest


def warp_pos(r, row, col):
    return r * 64 + ((row ^ (r & 1)) << 3) + (col ^ row)


def warp_res(k, R, swap):
    if not swap:
        return k
    r, k1, k2 = k % R, (k // R) & 7, k // (8 * R)
    return r * 8 + k1 + 8 * R * k2


def warp_twiddles(R):
    """The shared-memory twiddle table of the schedule, from wn^e."""
    N = 64 * R
    B = (R - 1) * 64
    w = np.exp(-2j * np.pi * np.arange(N) / N)
    idx = [((e & 63) * ((e >> 6) + 1)) % N if e < B else (R * (e & 7) * ((e - B) >> 3)) % N for e in range(N)]
    return w[np.array(idx)]


def dft(u):
    n = len(u)
    k = np.arange(n)
    return np.exp(-2j * np.pi * np.outer(k, k) / n) @ u


def fft_warp(z, R, swap):
    """The three passes of one warp over one complex sequence of 64 R."""
    N = 64 * R
    tw = warp_twiddles(R)
    work = np.zeros(N, complex)
    # Pass 1: radix R over stride 64.
    for i in range(64):
        u = dft(np.array([z[i + 64 * b] for b in range(R)]))
        for r in range(1, R):
            u[r] *= tw[(r - 1) * 64 + i]
        for r in range(R):
            work[warp_pos(r, i >> 3, i & 7)] = u[r]
    # Pass 2: radix 8 over m, twiddles w64^(t k1), in place.
    for pp in range(8 * R):
        r, t = pp >> 3, pp & 7
        a = dft(np.array([work[warp_pos(r, m, t)] for m in range(8)]))
        for k1 in range(1, 8):
            a[k1] *= tw[(R - 1) * 64 + k1 * 8 + t]
        for k1 in range(8):
            work[warp_pos(r, k1, t)] = a[k1]
    # Pass 3: radix 8 over t.
    out = np.zeros(N, complex)
    for pp in range(8 * R):
        r, k1 = pp >> 3, pp & 7
        a = dft(np.array([work[warp_pos(r, k1, t)] for t in range(8)]))
        for k2 in range(8):
            out[pp + 8 * R * k2 if swap else r + R * k1 + 8 * R * k2] = a[k2]
    return out


@pytest.mark.parametrize("R", [2, 4, 8])
def test_warp_positions_are_a_permutation(R):
    pos = sorted(warp_pos(r, row, col) for r in range(R) for row in range(8) for col in range(8))
    assert pos == list(range(64 * R))
    for swap in (False, True):
        assert sorted(warp_res(k, R, swap) for k in range(64 * R)) == list(range(64 * R))


def test_warp_rows_and_columns_hit_distinct_banks():
    """Eight lanes reading one row or one column of a sub-block (8-byte
    elements, 32 banks of 4 bytes) touch 16 distinct banks."""
    for r in range(8):
        for fixed in range(8):
            row = [2 * warp_pos(r, fixed, c) % 32 for c in range(8)]
            col = [2 * warp_pos(r, c, fixed) % 32 for c in range(8)]
            assert len(set(row)) == 8 and len(set(col)) == 8


@pytest.mark.parametrize("swap", [False, True])
@pytest.mark.parametrize("R", [2, 4, 8])
def test_warp_schedule_is_the_dft(R, swap):
    rng = np.random.default_rng(R)
    N = 64 * R
    z = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    got = fft_warp(z, R, swap)
    X = np.fft.fft(z)
    res = np.array([got[warp_res(k, R, swap)] for k in range(N)])
    assert np.abs(res - X).max() <= 1e-11 * np.abs(X).max()


def tdma_tables(lam, dz2, a, c):
    """den, s, g, h of the rescaled recurrence for one column group (the
    non-mean modes: Neumann top row), as k_tdma_table builds them."""
    kt = len(dz2)
    b = dz2 * lam - (a + c)
    b[0] += a[0]
    b[-1] += c[-1]
    den = np.empty(kt)
    den[0] = b[0]
    for k in range(1, kt):
        den[k] = b[k] - a[k] * (c[k - 1] / den[k - 1])
    s = dz2 / den
    g = np.zeros(kt)
    h = np.zeros(kt)
    g[1:] = a[1:] * s[:-1] / dz2[1:]
    h[:-1] = c[:-1] * s[1:] / dz2[:-1]
    return g, h, s


def sweeps(p, g, h, s, dtype):
    kt = len(p)
    z = np.empty(kt, dtype)
    acc = dtype(0)
    gd, hd, sd, pd = g.astype(dtype), h.astype(dtype), s.astype(dtype), p.astype(dtype)
    for k in range(kt):
        acc = dtype(pd[k] - gd[k] * acc)
        z[k] = acc
    x = np.empty(kt, dtype)
    xi = z[-1]
    x[-1] = sd[-1] * xi
    for k in range(kt - 2, -1, -1):
        xi = dtype(z[k] - hd[k] * xi)
        x[k] = dtype(sd[k] * xi)
    return x


def test_float_sweeps_within_the_stated_bound():
    """Groups whose forward coefficients stay at or below 0.999 (the float
    criterion of k_tdma_table) solve in float within 16 float ulps of the
    column's largest value; 256 uniform 15.6 m levels under 50 m spacing,
    the benchmark's grid."""
    kt, itot, dx, dz = 256, 512, 50., 4000. / 256
    dz2 = np.full(kt, dz * dz)
    a = np.ones(kt)
    c = np.ones(kt)
    a[0] = 0.
    c[-1] = 0.
    rng = np.random.default_rng(7)
    worst, checked = 0., 0
    for i in (8, 12, 20, 50, 100, 256):
        lam = 2. * (np.cos(2. * np.pi * i / itot) - 1.) / dx ** 2
        g, h, s = tdma_tables(lam, dz2, a, c)
        if np.abs(g).max() > 0.999:
            continue
        checked += 1
        for _ in range(4):
            p = rng.standard_normal(kt)
            x64 = sweeps(p, g, h, s, np.float64)
            x32 = sweeps(p, g, h, s, np.float32).astype(np.float64)
            worst = max(worst, np.abs(x32 - x64).max() / np.abs(x64).max())
    assert checked >= 5
    assert worst <= 16 * 2. ** -24, worst

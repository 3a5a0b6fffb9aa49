"""Case descriptions (microhh_gb300/cases.py): the reference-style .ini text
and the ghost layout, including the buffer layer and the flux limiter."""
import numpy as np

from microhh_gb300 import cases


def ini_items(text):
    """group -> {key: value} of the .ini text."""
    out, group = {}, None
    for line in text.splitlines():
        line = line.strip()
        if line.startswith("[") and line.endswith("]"):
            group = line[1:-1]
            out[group] = {}
        elif "=" in line and group:
            k, v = line.split("=", 1)
            out[group][k] = v
    return out


def test_ini_of_the_dry_cbl():
    c = cases.drycbl(32, 24, 16, 3200., 2400., 1600., seed=1)
    ini = ini_items(c.to_ini())
    assert ini["grid"]["itot"] == "32" and ini["grid"]["jtot"] == "24" and ini["grid"]["ktot"] == "16"
    assert ini["advec"]["swadvec"] == "2i5" and ini["diff"]["swdiff"] == "smag2"
    assert "buffer" not in ini and "fluxlimit_list" not in ini["advec"]


def test_buffer_and_flux_limiter_in_the_ini():
    c = cases.drycbl(32, 24, 16, 3200., 2400., 1600., seed=1)
    c.swbuffer, c.buffer_zstart, c.buffer_sigma, c.buffer_beta = True, 1000., 0.01, 2.
    c.fluxlimit = True
    ini = ini_items(c.to_ini())
    assert ini["buffer"] == {"swbuffer": "true", "zstart": "1000.0", "sigma": "0.01", "beta": "2.0"}
    assert ini["advec"]["fluxlimit_list"] == "th"


def test_ghost_layout_follows_the_vertical_ghost_cells():
    c = cases.drycbl(16, 12, 10, 1600., 1200., 1000., seed=2)
    assert c.igc == 3 and c.kgc == 1 and c.ghost_shape() == (12, 18, 22)
    c.fluxlimit = True
    # Advec_2i5 with a flux-limited scalar asks for two vertical ghost levels.
    assert c.kgc == 2 and c.ghost_shape() == (14, 18, 22)
    th = c.fields["th"]
    full = c.embed(th)
    assert np.array_equal(c.interior(full), th)
    assert np.all(full[:2] == 0.) and np.all(full[-2:] == 0.)


def test_buffer_profiles_are_the_initial_means():
    c = cases.drycbl(16, 12, 10, 1600., 1200., 1000., seed=3, noise_z=1000.)
    c.swbuffer = True
    for limited in (False, True):
        c.fluxlimit = limited
        prof = c.buffer_profiles()
        kg = c.kgc
        assert set(prof) == {"u", "v", "th"}
        assert prof["th"].shape == (c.ktot + 2 * kg,)
        assert np.allclose(prof["th"][kg:kg + c.ktot], c.fields["th"].mean(axis=(1, 2)))
        assert np.all(prof["th"][:kg] == 0.) and np.all(prof["th"][kg + c.ktot:] == 0.)

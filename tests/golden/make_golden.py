"""Generates the golden fixtures of the LES/DNS time step.

The fixtures are produced by the reference's own hot-path sources
(Advec_2i5, Advec_2, Diff_smag2, Diff_2, Pres_2, Timeloop, Boundary_cyclic,
Boundary_surface, Buffer, the flux limiter of advec_monotonic.h), compiled unchanged into oracle/_ref/libmhh_ref.so by
``make -C oracle ref`` (which needs the MicroHH source tree).  Each fixture
holds the seeded initial fields and the fields and diagnostics after one RK3
step (three substeps), so that the CPU restatement in oracle/ and the CUDA
path can both be checked against the reference without the reference tree.

Run from the repository root:  python tests/golden/make_golden.py [name ...]
(no names: every fixture).
"""
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from microhh_gb300 import cases  # noqa: E402
from oracle import orcpy  # noqa: E402


def golden_cases():
    """The fixture cases: name -> Case."""
    out = {}
    out["cbl_surface_16x12x10"] = cases.drycbl(16, 12, 10, 1600., 1200., 1000., seed=11, noise_z=400.)
    c = cases.drycbl(12, 20, 8, 1200., 2000., 800., seed=12, noise_z=300., sbot=0.2)
    c.name = "cbl_surface_12x20x8"
    out[c.name] = c
    c = cases.drycbl(16, 12, 10, 1600., 1200., 1000., seed=13, surface=False, noise_z=400.)
    c.sbcbot, c.sbot = cases.BC_DIRICHLET, 301.0
    c.name = "cbl_walls_16x12x10"
    out[c.name] = c
    c = cases.drycbl(16, 16, 12, 1600., 1600., 1200., seed=14, noise_z=600.)
    c.thermo = False
    rng = np.random.Generator(np.random.PCG64(14))
    c.fields = {"u": 2.0 + 0.5 * rng.standard_normal((12, 16, 16)),
                "v": -1.0 + 0.5 * rng.standard_normal((12, 16, 16)),
                "w": 0.1 * rng.standard_normal((12, 16, 16))}
    c.fields["w"][0] = 0.0
    c.name = "neutral_surface_16x16x12"
    out[c.name] = c
    c = cases.channel(16, 12, 10, seed=15, dt=1e-3, adaptivestep=True)
    c.name = "channel_16x12x10"
    out[c.name] = c
    # Buffer layer (src/buffer.cxx) over the top third, with a mean wind and
    # perturbations at every level so that every field is relaxed.
    c = cases.drycbl(16, 12, 12, 1600., 1200., 1200., seed=16, noise_z=1200.)
    rng = np.random.Generator(np.random.PCG64(16))
    c.fields["u"] = 2.0 + 0.02 * np.arange(12)[:, None, None] + 0.3 * rng.standard_normal((12, 12, 16))
    c.fields["v"] = -1.0 + 0.3 * rng.standard_normal((12, 12, 16))
    c.fields["w"] = 0.1 * rng.standard_normal((12, 12, 16))
    c.fields["w"][0] = 0.0
    c.swbuffer, c.buffer_zstart, c.buffer_sigma, c.buffer_beta = True, 800., 0.01, 2.
    c.name = "cbl_buffer_16x12x12"
    out[c.name] = c
    # th advected with the flux limiter (src/advec_2i5.cxx fluxlimit_list;
    # two vertical ghost levels), with sharp theta fronts so that the
    # limiter is active.
    c = cases.drycbl(16, 12, 12, 1600., 1200., 1200., seed=17, noise_z=1200., noise=0.5)
    rng = np.random.Generator(np.random.PCG64(17))
    c.fields["u"] = 2.0 + 0.5 * rng.standard_normal((12, 12, 16))
    c.fields["v"] = -1.0 + 0.5 * rng.standard_normal((12, 12, 16))
    c.fields["w"] = 0.3 * rng.standard_normal((12, 12, 16))
    c.fields["w"][0] = 0.0
    c.fields["th"][:, :, 8:] += 1.0
    c.fluxlimit = True
    c.name = "cbl_fluxlimit_16x12x12"
    out[c.name] = c
    return out


DIAG = ("cfl", "dn", "div")


def run_reference(case, ref=True):
    m = orcpy.model_from_case(case, ref=ref)
    m.run_substeps(3)
    res = {}
    names = case.prognostic_names() + ["p"] + (["evisc"] if case.diff == "smag2" else [])
    for n in names:
        res["out_" + n] = m.get(n)
    # The status diagnostics run after the periodic and wall ghost-cell fill
    # of the next substep (src/model.cxx:367-382).
    m.lib.orc_set_cyclic_and_ghost(m.h)
    for n in DIAG:
        res["diag_" + n] = np.float64(getattr(m, n)())
    res["diag_dt"] = np.float64(m.dt())
    m.close()
    return res


def main():
    orcpy.build(ref=True)
    here = os.path.dirname(os.path.abspath(__file__))
    only = set(sys.argv[1:])
    for name, case in golden_cases().items():
        if only and name not in only:
            continue
        res = run_reference(case)
        for n in case.prognostic_names():
            res["in_" + n] = case.embed(case.fields[n])
        if case.swbuffer:
            for n, prof in case.buffer_profiles().items():
                res["buf_" + n] = prof
        path = os.path.join(here, name + ".npz")
        np.savez_compressed(path, **res)
        print("wrote", path, os.path.getsize(path))


if __name__ == "__main__":
    main()

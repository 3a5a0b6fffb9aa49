"""Seeded synthetic cases for the LES/DNS time step.

Each case is a plain description -- grid, physics switches, time step and the
initial prognostic fields -- from which both the .ini text of the C++ host
(microhh_gb300.model) and the test oracle are configured.  Initial noise uses
numpy's PCG64 generator, which gives the same numbers on every platform (the
reference seeds glibc ``std::rand`` per MPI rank, src/fields.cxx:1035-1080,
which is not portable, so the fields are injected instead).

Cases:
  * ``drycbl``  -- dry convective boundary layer LES (Advec_2i5, Smagorinsky,
    Monin-Obukhov surface, Boussinesq thermodynamics), after
    cases/drycblles/drycblles.ini.
  * ``channel`` -- turbulent channel DNS (Advec_2, Diff_2, constant pressure
    gradient, stretched wall-normal grid), after cases/moser180.
"""
from dataclasses import dataclass, field
import math

import numpy as np

BC_DIRICHLET, BC_NEUMANN, BC_FLUX = 0, 1, 2
MBC_NAMES = {BC_DIRICHLET: "noslip", BC_NEUMANN: "freeslip"}
SBC_NAMES = {BC_DIRICHLET: "dirichlet", BC_NEUMANN: "neumann", BC_FLUX: "flux"}


@dataclass
class Case:
    name: str
    itot: int
    jtot: int
    ktot: int
    xsize: float
    ysize: float
    zsize: float
    z: np.ndarray                      # ktot full-level heights
    advec: str = "2i5"                 # "2i5" | "2"
    diff: str = "smag2"                # "smag2" | "2"
    thermo: bool = True                # dry Boussinesq with prognostic th
    surface: bool = True               # swboundary = surface (MOST)
    mbcbot: int = BC_DIRICHLET
    mbctop: int = BC_NEUMANN
    sbcbot: int = BC_FLUX
    sbctop: int = BC_NEUMANN
    ubot: float = 0.0
    utop: float = 0.0
    vbot: float = 0.0
    vtop: float = 0.0
    sbot: float = 0.1
    stop: float = 0.003
    visc: float = 1.e-5
    svisc: float = 1.e-5
    cs: float = 0.23
    tpr: float = 1.0 / 3.0
    dnmax: float = 0.4
    swmason: bool = True
    cflmax: float = 1.2
    thref0: float = 300.0
    swlspres: bool = False
    dpdx: float = 0.0
    z0m: float = 0.1
    z0h: float = 0.1
    dt: float = 2.0
    dtmax: float = 0.0
    adaptivestep: bool = False
    swbuffer: bool = False             # [buffer] damping layer above buffer_zstart
    buffer_zstart: float = 0.0
    buffer_sigma: float = 2.0
    buffer_beta: float = 2.0
    fluxlimit: bool = False            # [advec] fluxlimit_list=th (Advec_2i5 only)
    fields: dict = field(default_factory=dict)   # name -> (ktot, jtot, itot) float64

    @property
    def igc(self):
        return 3 if self.advec == "2i5" else 1

    @property
    def kgc(self):
        # Advec_2i5 with a flux-limited scalar asks for two vertical ghost
        # levels (src/advec_2i5.cxx:36-46).
        return 2 if self.advec == "2i5" and self.fluxlimit else 1

    @property
    def ncells_interior(self):
        return self.itot * self.jtot * self.ktot

    def ghost_shape(self):
        g = self.igc
        return (self.ktot + 2 * self.kgc, self.jtot + 2 * g, self.itot + 2 * g)

    def embed(self, interior):
        """Places an interior (ktot, jtot, itot) array into a zeroed ghost layout."""
        g, kg = self.igc, self.kgc
        out = np.zeros(self.ghost_shape(), dtype=np.float64)
        out[kg:kg + self.ktot, g:g + self.jtot, g:g + self.itot] = interior
        return out

    def interior(self, full):
        g, kg = self.igc, self.kgc
        return full[kg:kg + self.ktot, g:g + self.jtot, g:g + self.itot]

    def prognostic_names(self):
        return ["u", "v", "w"] + (["th"] if self.thermo else [])

    def to_ini(self):
        """The reference-style .ini text for this case."""
        f = repr
        lines = [
            "[master]", "npx=1", "npy=1", "",
            "[grid]", f"itot={self.itot}", f"jtot={self.jtot}", f"ktot={self.ktot}",
            f"xsize={f(self.xsize)}", f"ysize={f(self.ysize)}", f"zsize={f(self.zsize)}",
            "swspatialorder=2", "",
            "[advec]", f"swadvec={self.advec}", f"cflmax={f(self.cflmax)}",
            *(["fluxlimit_list=th"] if self.fluxlimit else []), "",
            "[diff]", f"swdiff={self.diff}", f"cs={f(self.cs)}", f"tPr={f(self.tpr)}",
            f"dnmax={f(self.dnmax)}", f"swmason={'true' if self.swmason else 'false'}", "",
            "[thermo]", f"swthermo={'dry' if self.thermo else '0'}", "swbasestate=boussinesq",
            f"thref0={f(self.thref0)}", "pbot=100000.", "",
            "[force]", f"swlspres={'dpdx' if self.swlspres else '0'}", f"dpdx={f(self.dpdx)}", "",
            "[boundary]", f"swboundary={'surface' if self.surface else 'default'}",
            f"mbcbot={MBC_NAMES[self.mbcbot]}", f"mbctop={MBC_NAMES[self.mbctop]}",
            f"ubot={f(self.ubot)}", f"utop={f(self.utop)}", f"vbot={f(self.vbot)}", f"vtop={f(self.vtop)}",
            f"sbcbot={SBC_NAMES[self.sbcbot]}", f"sbctop={SBC_NAMES[self.sbctop]}",
            f"sbot={f(self.sbot)}", f"stop={f(self.stop)}",
            f"z0m={f(self.z0m)}", f"z0h={f(self.z0h)}", "",
            "[fields]", f"visc={f(self.visc)}", f"svisc={f(self.svisc)}", "",
            "[pres]", "swpres=2", "",
            "[time]", "starttime=0", "endtime=1e12", "savetime=1e9", f"dt={f(self.dt)}",
        ]
        if self.dtmax > 0:
            lines.append(f"dtmax={f(self.dtmax)}")
        lines += [f"adaptivestep={'true' if self.adaptivestep else 'false'}", "rkorder=3", ""]
        if self.swbuffer:
            lines += ["[buffer]", "swbuffer=true", f"zstart={f(self.buffer_zstart)}",
                      f"sigma={f(self.buffer_sigma)}", f"beta={f(self.buffer_beta)}", ""]
        return "\n".join(lines)

    def buffer_profiles(self):
        """The relaxation targets of the buffer layer: the horizontal means of
        the initial u, v and th (the reference reads the case's initial
        profiles), as kcells arrays with zero ghost levels."""
        out = {}
        for n in ("u", "v", "th"):
            if n in self.fields:
                prof = np.zeros(self.ktot + 2 * self.kgc)
                prof[self.kgc:self.kgc + self.ktot] = self.fields[n].mean(axis=(1, 2))
                out[n] = prof
        return out


def uniform_z(ktot, zsize):
    dz = zsize / ktot
    return (np.arange(ktot) + 0.5) * dz


def drycbl(itot=64, jtot=64, ktot=64, xsize=6400., ysize=6400., zsize=4000., seed=0,
           sbot=0.1, lapse=0.003, surface=True, dt=2.0, noise=0.1, noise_z=200., name=None):
    """Dry convective boundary layer LES.

    theta = 300 K below 1000 m, then + lapse K/m; u = v = w = 0; uniform
    theta noise of amplitude ``noise`` K in the lowest ``noise_z`` m.
    """
    z = uniform_z(ktot, zsize)
    rng = np.random.Generator(np.random.PCG64(seed))
    th_prof = np.where(z < 1000., 300., 300. + lapse * (z - 1000.))
    th = np.broadcast_to(th_prof[:, None, None], (ktot, jtot, itot)).copy()
    mask = z < noise_z
    th[mask] += rng.uniform(-noise, noise, size=(int(mask.sum()), jtot, itot))
    zeros = np.zeros((ktot, jtot, itot))
    return Case(
        name=name or f"drycbl_{itot}x{jtot}x{ktot}", itot=itot, jtot=jtot, ktot=ktot,
        xsize=xsize, ysize=ysize, zsize=zsize, z=z,
        advec="2i5", diff="smag2", thermo=True, surface=surface,
        mbcbot=BC_DIRICHLET, mbctop=BC_NEUMANN, sbcbot=BC_FLUX, sbctop=BC_NEUMANN,
        sbot=sbot, stop=lapse, visc=1.e-5, svisc=1.e-5, cs=0.23, tpr=1. / 3., swmason=True,
        thref0=300., z0m=0.1, z0h=0.1, dt=dt, adaptivestep=False,
        fields={"u": zeros.copy(), "v": zeros.copy(), "w": zeros.copy(), "th": th})


def stretched_channel_z(ktot, gamma=2.75):
    """Wall-normal levels of a 2-high channel, tanh-stretched towards both walls.

    Half levels are zh_k = 1 + tanh(gamma (2k/ktot - 1)) / tanh(gamma),
    k = 0..ktot (zh_0 = 0, zh_ktot = 2); full levels are their midpoints.
    """
    k = np.arange(ktot + 1)
    zh = 1.0 + np.tanh(gamma * (2.0 * k / ktot - 1.0)) / math.tanh(gamma)
    zh[0], zh[-1] = 0.0, 2.0
    return 0.5 * (zh[1:] + zh[:-1])


def channel(itot=256, jtot=192, ktot=128, seed=1, gamma=2.75, ubulk=None, noise=0.05,
            dt=1.e-3, adaptivestep=True, name=None):
    """Turbulent channel DNS at Re_tau ~ 180 (u_tau = 1, h = 1, nu = 1/180).

    u = parabolic laminar profile with bulk velocity ``ubulk`` (default the
    turbulent bulk velocity ~15.6 u_tau at Re_tau 180) plus Gaussian noise of
    ``noise`` * ubulk in u, v and w.
    """
    xsize, ysize, zsize = 2. * math.pi, math.pi, 2.
    z = stretched_channel_z(ktot, gamma)
    rng = np.random.Generator(np.random.PCG64(seed))
    ub = 15.6 if ubulk is None else ubulk
    uprof = 1.5 * ub * (1. - (z - 1.) ** 2)
    u = np.broadcast_to(uprof[:, None, None], (ktot, jtot, itot)).copy()
    sh = (ktot, jtot, itot)
    u += rng.normal(0., noise * ub, size=sh)
    v = rng.normal(0., noise * ub, size=sh)
    w = rng.normal(0., noise * ub, size=sh)
    w[0] = 0.0   # w sits on the wall at the first half level
    return Case(
        name=name or f"channel_{itot}x{jtot}x{ktot}", itot=itot, jtot=jtot, ktot=ktot,
        xsize=xsize, ysize=ysize, zsize=zsize, z=z,
        advec="2", diff="2", thermo=False, surface=False,
        mbcbot=BC_DIRICHLET, mbctop=BC_DIRICHLET, sbcbot=BC_FLUX, sbctop=BC_FLUX,
        sbot=0., stop=0., visc=1. / 180., svisc=1. / 180., cflmax=1.2, dnmax=0.4,
        swlspres=True, dpdx=-1.0, dt=dt, dtmax=0.0, adaptivestep=adaptivestep,
        fields={"u": u, "v": v, "w": w})

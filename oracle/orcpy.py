"""ctypes binding of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Loads either the C restatement (oracle/libmhh_oracle.so) or the reference
build (oracle/_ref/libmhh_ref.so, built from the reference's own sources by
``make ref``); both export the C API of oracle/mhh_oracle.h.  Only the tests,
``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_ORACLE = os.path.join(HERE, "libmhh_oracle.so")
LIB_REF = os.path.join(HERE, "_ref", "libmhh_ref.so")

ADVEC_2, ADVEC_2I5 = 2, 25
DIFF_2, DIFF_SMAG2 = 2, 7
BC_DIRICHLET, BC_NEUMANN, BC_FLUX = 0, 1, 2


class Params(ctypes.Structure):
    _fields_ = [
        ("itot", ctypes.c_int), ("jtot", ctypes.c_int), ("ktot", ctypes.c_int),
        ("xsize", ctypes.c_double), ("ysize", ctypes.c_double), ("zsize", ctypes.c_double),
        ("advec", ctypes.c_int), ("diff", ctypes.c_int), ("thermo", ctypes.c_int), ("surface", ctypes.c_int),
        ("mbcbot", ctypes.c_int), ("mbctop", ctypes.c_int), ("sbcbot", ctypes.c_int), ("sbctop", ctypes.c_int),
        ("ubot", ctypes.c_double), ("utop", ctypes.c_double), ("vbot", ctypes.c_double), ("vtop", ctypes.c_double),
        ("sbot", ctypes.c_double), ("stop", ctypes.c_double),
        ("visc", ctypes.c_double), ("svisc", ctypes.c_double),
        ("cs", ctypes.c_double), ("tpr", ctypes.c_double), ("dnmax", ctypes.c_double),
        ("swmason", ctypes.c_int),
        ("cflmax", ctypes.c_double), ("thref0", ctypes.c_double),
        ("swlspres", ctypes.c_int), ("dpdx", ctypes.c_double),
        ("z0m", ctypes.c_double), ("z0h", ctypes.c_double),
        ("dt", ctypes.c_double), ("dtmax", ctypes.c_double), ("adaptivestep", ctypes.c_int),
        ("swbuffer", ctypes.c_int), ("buf_zstart", ctypes.c_double), ("buf_sigma", ctypes.c_double),
        ("buf_beta", ctypes.c_double), ("fluxlimit_s", ctypes.c_int),
    ]


def build(ref=False):
    """Builds the restatement (and with ref=True the reference build)."""
    subprocess.run(["make", "-s", "-C", HERE] + (["ref"] if ref else []), check=True)


_libs = {}


def load(ref=False):
    path = LIB_REF if ref else LIB_ORACLE
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise FileNotFoundError(path)
    lib = ctypes.CDLL(path)
    P = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    lib.orc_create.restype = P
    lib.orc_create.argtypes = [ctypes.POINTER(Params), dp]
    lib.orc_destroy.argtypes = [P]
    lib.orc_ncells.restype = ctypes.c_long
    lib.orc_ncells.argtypes = [P]
    lib.orc_dims.argtypes = [P, ctypes.POINTER(ctypes.c_int)]
    for fn in ("orc_set_field", "orc_get_field", "orc_get_profile", "orc_get_2d"):
        getattr(lib, fn).restype = ctypes.c_int
        getattr(lib, fn).argtypes = [P, ctypes.c_char_p, dp]
    lib.orc_run_substeps.argtypes = [P, ctypes.c_int]
    for fn in ("orc_get_cfl", "orc_get_dn", "orc_get_div"):
        getattr(lib, fn).restype = ctypes.c_double
        getattr(lib, fn).argtypes = [P]
    lib.orc_get_dt.restype = ctypes.c_double
    lib.orc_get_dt.argtypes = [P]
    lib.orc_get_substep.restype = ctypes.c_int
    lib.orc_get_substep.argtypes = [P]
    lib.orc_get_itime.restype = ctypes.c_ulong
    lib.orc_get_itime.argtypes = [P]
    for fn in ("orc_set_cyclic_and_ghost", "orc_exec_viscosity", "orc_exec_thermo", "orc_exec_boundary",
               "orc_exec_advec", "orc_exec_diff", "orc_exec_force", "orc_exec_timeloop", "orc_exec_buffer"):
        getattr(lib, fn).argtypes = [P]
    lib.orc_set_buffer_profile.restype = ctypes.c_int
    lib.orc_set_buffer_profile.argtypes = [P, ctypes.c_char_p, dp]
    lib.orc_exec_pres.argtypes = [P, ctypes.c_double]
    for fn in ("orc_r2hc", "orc_hc2r"):
        getattr(lib, fn).argtypes = [ctypes.c_int, ctypes.c_int, dp, ctypes.c_long, ctypes.c_long]
    lib.orc_num_threads.restype = ctypes.c_int
    _libs[path] = lib
    return lib


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Model:
    """One oracle model instance (restatement or reference build)."""

    FIELDS = ("u", "v", "w", "th", "ut", "vt", "wt", "tht", "p", "evisc")

    def __init__(self, params, z, ref=False):
        self.lib = load(ref)
        self.params = params
        self._z = np.ascontiguousarray(z, dtype=np.float64)
        self.h = self.lib.orc_create(ctypes.byref(params), _dptr(self._z))
        d = (ctypes.c_int * 6)()
        self.lib.orc_dims(self.h, d)
        self.igc, self.jgc, self.kgc, self.icells, self.jcells, self.kcells = list(d)
        self.shape = (self.kcells, self.jcells, self.icells)

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.shape)
        if self.lib.orc_set_field(self.h, name.encode(), _dptr(a)) != 0:
            raise KeyError(name)

    def get(self, name):
        a = np.empty(self.shape, dtype=np.float64)
        if self.lib.orc_get_field(self.h, name.encode(), _dptr(a)) != 0:
            raise KeyError(name)
        return a

    def set_buffer_profile(self, name, prof):
        a = np.ascontiguousarray(prof, dtype=np.float64)
        if self.lib.orc_set_buffer_profile(self.h, name.encode(), _dptr(a)) != 0:
            raise KeyError(name)

    def profile(self, name):
        a = np.empty(self.kcells, dtype=np.float64)
        if self.lib.orc_get_profile(self.h, name.encode(), _dptr(a)) != 0:
            raise KeyError(name)
        return a

    def surface(self, name):
        a = np.empty((self.jcells, self.icells), dtype=np.float64)
        if self.lib.orc_get_2d(self.h, name.encode(), _dptr(a)) != 0:
            raise KeyError(name)
        return a

    def run_substeps(self, n):
        self.lib.orc_run_substeps(self.h, n)

    def cfl(self):
        return self.lib.orc_get_cfl(self.h)

    def dn(self):
        return self.lib.orc_get_dn(self.h)

    def div(self):
        return self.lib.orc_get_div(self.h)

    def dt(self):
        return self.lib.orc_get_dt(self.h)

    def substep(self):
        return self.lib.orc_get_substep(self.h)


def r2hc(x, ref=False):
    """Halfcomplex transform along the last axis (copy)."""
    lib = load(ref)
    a = np.ascontiguousarray(x, dtype=np.float64).copy()
    n = a.shape[-1]
    lib.orc_r2hc(n, a.size // n, _dptr(a), 1, n)
    return a


def hc2r(x, ref=False):
    lib = load(ref)
    a = np.ascontiguousarray(x, dtype=np.float64).copy()
    n = a.shape[-1]
    lib.orc_hc2r(n, a.size // n, _dptr(a), 1, n)
    return a


def params_from_case(case):
    """Oracle parameters for a microhh_gb300.cases.Case."""
    p = Params()
    p.itot, p.jtot, p.ktot = case.itot, case.jtot, case.ktot
    p.xsize, p.ysize, p.zsize = case.xsize, case.ysize, case.zsize
    p.advec = ADVEC_2I5 if case.advec == "2i5" else ADVEC_2
    p.diff = DIFF_SMAG2 if case.diff == "smag2" else DIFF_2
    p.thermo = 1 if case.thermo else 0
    p.surface = 1 if case.surface else 0
    p.mbcbot, p.mbctop, p.sbcbot, p.sbctop = case.mbcbot, case.mbctop, case.sbcbot, case.sbctop
    p.ubot, p.utop, p.vbot, p.vtop = case.ubot, case.utop, case.vbot, case.vtop
    p.sbot, p.stop = case.sbot, case.stop
    p.visc, p.svisc = case.visc, case.svisc
    p.cs, p.tpr, p.dnmax = case.cs, case.tpr, case.dnmax
    p.swmason = 1 if case.swmason else 0
    p.cflmax, p.thref0 = case.cflmax, case.thref0
    p.swlspres = 1 if case.swlspres else 0
    p.dpdx = case.dpdx
    p.z0m, p.z0h = case.z0m, case.z0h
    p.dt, p.dtmax = case.dt, case.dtmax
    p.adaptivestep = 1 if case.adaptivestep else 0
    p.swbuffer = 1 if case.swbuffer else 0
    p.buf_zstart, p.buf_sigma, p.buf_beta = case.buffer_zstart, case.buffer_sigma, case.buffer_beta
    p.fluxlimit_s = 1 if case.fluxlimit else 0
    return p


def model_from_case(case, ref=False):
    """An oracle model loaded with the case's initial fields."""
    m = Model(params_from_case(case), case.z, ref=ref)
    for name in case.prognostic_names():
        m.set(name, case.embed(case.fields[name]))
    if case.swbuffer:
        for name, prof in case.buffer_profiles().items():
            m.set_buffer_profile(name, prof)
    return m

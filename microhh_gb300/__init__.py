"""GB300-native LES/DNS time step of MicroHH: Python bindings.

The arithmetic lives in the sm_103a CUDA kernels of lib/libmhh_gb300.so
(C-ABI: include/mhh.h) driven by the C++ host layer in lib/libmhh_host.so
(include/mhh_model.h).  This module only binds them with ctypes; there is no
Python or CPU fallback -- importing the bindings without the built libraries
raises.
"""
import ctypes
import os

import numpy as np

from . import cases  # noqa: F401

PKG = os.path.dirname(os.path.abspath(__file__))
LIBDIR = os.path.join(PKG, "lib")

FP64, FP32 = 64, 32
# mhh_status codes of include/mhh.h used by callers.
ERR_ARG, ERR_NONFINITE = -1, -4
ADVEC_2, ADVEC_2I5 = 2, 25
DIFF_NONE, DIFF_2, DIFF_SMAG2 = 0, 2, 7


class MhhError(RuntimeError):
    """A failed entry point; ``status`` is its mhh_status code (include/mhh.h),
    e.g. -4 (MHH_ERR_NONFINITE) for a run with non-finite numbers."""

    def __init__(self, msg, status=None):
        super().__init__(msg)
        self.status = status


class GridDesc(ctypes.Structure):
    _fields_ = [("itot", ctypes.c_int), ("jtot", ctypes.c_int), ("ktot", ctypes.c_int),
                ("igc", ctypes.c_int), ("jgc", ctypes.c_int), ("kgc", ctypes.c_int),
                ("xsize", ctypes.c_double), ("ysize", ctypes.c_double), ("zsize", ctypes.c_double)]


class Grid(ctypes.Structure):
    _fields_ = [("itot", ctypes.c_int), ("jtot", ctypes.c_int), ("ktot", ctypes.c_int),
                ("igc", ctypes.c_int), ("jgc", ctypes.c_int), ("kgc", ctypes.c_int),
                ("icells", ctypes.c_int), ("jcells", ctypes.c_int), ("kcells", ctypes.c_int),
                ("ijcells", ctypes.c_int),
                ("istart", ctypes.c_int), ("iend", ctypes.c_int), ("jstart", ctypes.c_int),
                ("jend", ctypes.c_int), ("kstart", ctypes.c_int), ("kend", ctypes.c_int),
                ("ncells", ctypes.c_longlong), ("dx", ctypes.c_double), ("dy", ctypes.c_double),
                ("zsize", ctypes.c_double), ("precision", ctypes.c_int)]


class Physics(ctypes.Structure):
    _fields_ = [("visc", ctypes.c_double), ("svisc", ctypes.c_double),
                ("cs", ctypes.c_double), ("tpr", ctypes.c_double), ("dnmax", ctypes.c_double),
                ("swmason", ctypes.c_int), ("cflmax", ctypes.c_double), ("thref0", ctypes.c_double),
                ("thermo", ctypes.c_int), ("surface", ctypes.c_int),
                ("z0m", ctypes.c_double), ("z0h", ctypes.c_double)]


class Fields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ("u", "v", "w", "s", "ut", "vt", "wt", "st", "evisc", "p")]


class BcFields(ctypes.Structure):
    _fields_ = [(f"{f}_{k}", ctypes.c_void_p) for f in ("u", "v", "s")
                for k in ("bot", "top", "gradbot", "gradtop", "fluxbot", "fluxtop")]


class SubstepConfig(ctypes.Structure):
    _fields_ = [("advec", ctypes.c_int), ("diff", ctypes.c_int), ("swlspres", ctypes.c_int),
                ("dpdx", ctypes.c_double), ("mbcbot", ctypes.c_int), ("mbctop", ctypes.c_int),
                ("sbcbot", ctypes.c_int), ("sbctop", ctypes.c_int)]


_kern = None
_host = None


_last_call = [""]


def _note_call(result, func, args):
    _last_call[0] = func.__name__
    return result


def _declare(lib, name, restype, argtypes):
    f = getattr(lib, name)
    f.restype = restype
    f.argtypes = argtypes
    if restype is ctypes.c_int:
        f.errcheck = _note_call
    return f


def load():
    """Loads both native libraries (building them first if needed)."""
    global _kern, _host
    if _host is not None:
        return _kern, _host
    kpath = os.path.join(LIBDIR, "libmhh_gb300.so")
    hpath = os.path.join(LIBDIR, "libmhh_host.so")
    if not (os.path.exists(kpath) and os.path.exists(hpath)):
        from . import build
        build.build()
    kern = ctypes.CDLL(kpath, mode=ctypes.RTLD_GLOBAL)
    host = ctypes.CDLL(hpath)
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    dp = ctypes.POINTER(ctypes.c_double)
    S = ctypes.c_void_p  # cudaStream_t
    # C-ABI of the kernels (include/mhh.h)
    _declare(kern, "mhh_last_error", ctypes.c_char_p, [])
    _declare(kern, "mhh_launch_count", ctypes.c_longlong, [])
    _declare(kern, "mhh_set_option", I, [ctypes.c_char_p, I])
    _declare(kern, "mhh_timing_enable", I, [I])
    _declare(kern, "mhh_timing_reset", I, [])
    _declare(kern, "mhh_timing_collect", I, [])
    _declare(kern, "mhh_timing_count", I, [])
    _declare(kern, "mhh_timing_get", I, [I, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(ctypes.c_longlong), dp])
    _declare(kern, "mhh_ctx_create", I, [ctypes.POINTER(GridDesc), dp, I, ctypes.POINTER(Physics), ctypes.POINTER(P)])
    _declare(kern, "mhh_ctx_destroy", I, [P])
    _declare(kern, "mhh_ctx_get_grid", I, [P, ctypes.POINTER(Grid)])
    _declare(kern, "mhh_ctx_get_profile", I, [P, ctypes.c_char_p, dp])
    _declare(kern, "mhh_boundary_cyclic", I, [P, P, I, S])
    _declare(kern, "mhh_boundary_set_bc", I, [P, P, P, P, I, D, D, I, S])
    _declare(kern, "mhh_boundary_ghost_cells", I, [P, P, I, P, P, I, P, P, S])
    _declare(kern, "mhh_boundary_surface_exec", I, [P, ctypes.POINTER(Fields), ctypes.POINTER(BcFields), I, S])
    _declare(kern, "mhh_boundary_surface_init", I, [P, I])
    _declare(kern, "mhh_boundary_surface_get", I, [P, ctypes.c_char_p, dp])
    for n in ("mhh_advec_2i5_exec", "mhh_advec_2_exec", "mhh_diff_2_exec", "mhh_thermo_dry_exec"):
        _declare(kern, n, I, [P, ctypes.POINTER(Fields), S])
    _declare(kern, "mhh_advec_get_cfl", I, [P, I, ctypes.POINTER(Fields), D, dp, S])
    _declare(kern, "mhh_advec_get_time_limit", I, [P, I, ctypes.POINTER(Fields), ctypes.c_ulonglong, D,
                                                  ctypes.POINTER(ctypes.c_ulonglong), S])
    _declare(kern, "mhh_diff_smag2_exec_viscosity", I, [P, ctypes.POINTER(Fields), ctypes.POINTER(BcFields), S])
    _declare(kern, "mhh_diff_smag2_exec", I, [P, ctypes.POINTER(Fields), ctypes.POINTER(BcFields), S])
    _declare(kern, "mhh_diff_smag2_get_dn", I, [P, ctypes.POINTER(Fields), D, dp, S])
    _declare(kern, "mhh_diff_2_get_dn", I, [P, D, dp])
    _declare(kern, "mhh_force_dpdx_exec", I, [P, ctypes.POINTER(Fields), D, S])
    _declare(kern, "mhh_pres_2_exec", I, [P, ctypes.POINTER(Fields), D, S])
    _declare(kern, "mhh_pres_2_get_divergence", I, [P, ctypes.POINTER(Fields), dp, S])
    _declare(kern, "mhh_fft_forward", I, [P, P, S])
    _declare(kern, "mhh_fft_backward", I, [P, P, S])
    _declare(kern, "mhh_timeloop_rk3", I, [P, P, P, I, D, S])
    _declare(kern, "mhh_advec_2i5_set_fluxlimit", I, [P, I])
    _declare(kern, "mhh_buffer_setup", I, [P, D, D, D])
    _declare(kern, "mhh_buffer_set_profile", I, [P, ctypes.c_char_p, dp])
    _declare(kern, "mhh_buffer_exec", I, [P, ctypes.POINTER(Fields), S])
    _declare(kern, "mhh_substep_begin", I, [P, ctypes.POINTER(SubstepConfig), ctypes.POINTER(Fields),
                                           ctypes.POINTER(BcFields), S])
    _declare(kern, "mhh_substep_end", I, [P, ctypes.POINTER(SubstepConfig), ctypes.POINTER(Fields),
                                         ctypes.POINTER(BcFields), I, D, S])
    # Host layer (include/mhh_model.h)
    _declare(host, "mhh_model_last_error", ctypes.c_char_p, [])
    _declare(host, "mhh_model_create", I, [ctypes.c_char_p, dp, I, I, ctypes.POINTER(P)])
    _declare(host, "mhh_model_destroy", I, [P])
    _declare(host, "mhh_model_set_field", I, [P, ctypes.c_char_p, dp])
    _declare(host, "mhh_model_get_field", I, [P, ctypes.c_char_p, dp])
    _declare(host, "mhh_model_set_field_native", I, [P, ctypes.c_char_p, P])
    _declare(host, "mhh_model_get_field_native", I, [P, ctypes.c_char_p, P])
    _declare(host, "mhh_model_run_steps", I, [P, I, I])
    _declare(host, "mhh_model_run_substeps", I, [P, I, I])
    for n in ("mhh_model_get_cfl", "mhh_model_get_dn", "mhh_model_get_div", "mhh_model_get_dt", "mhh_model_get_time"):
        _declare(host, n, I, [P, dp])
    _declare(host, "mhh_model_get_substep", I, [P, ctypes.POINTER(ctypes.c_int)])
    _declare(host, "mhh_model_get_grid", I, [P, ctypes.POINTER(Grid)])
    _declare(host, "mhh_model_get_profile", I, [P, ctypes.c_char_p, dp])
    _declare(host, "mhh_model_get_surface", I, [P, ctypes.c_char_p, dp])
    _declare(host, "mhh_model_set_stream", I, [P, S])
    _declare(host, "mhh_model_set_buffer_profile", I, [P, ctypes.c_char_p, dp])
    _declare(host, "mhh_model_synchronize", I, [P])
    _declare(host, "mhh_model_get_device_fields", I, [P, ctypes.POINTER(Fields), ctypes.POINTER(BcFields)])
    _declare(host, "mhh_model_get_ctx", P, [P])
    _declare(host, "mhh_model_save", I, [P, ctypes.c_char_p, ctypes.POINTER(I)])
    _declare(host, "mhh_model_load", I, [P, ctypes.c_char_p, I])
    # Ensembles and the server (include/mhh_batch.h)
    _declare(host, "mhh_batch_last_error", ctypes.c_char_p, [])
    _declare(host, "mhh_ensemble_create", I, [ctypes.POINTER(P)])
    _declare(host, "mhh_ensemble_add", I, [P, P])
    _declare(host, "mhh_ensemble_autotune", I, [P, ctypes.c_char_p, I])
    _declare(host, "mhh_ensemble_run_steps", I, [P, I, I])
    _declare(host, "mhh_ensemble_synchronize", I, [P])
    _declare(host, "mhh_ensemble_destroy", I, [P])
    _declare(host, "mhh_server_create", I, [D, I, ctypes.POINTER(P)])
    _declare(host, "mhh_server_submit", I, [P, ctypes.c_char_p, dp, I, I, I, D, I, ctypes.POINTER(I)])
    _declare(host, "mhh_server_set_initial", I, [P, I, ctypes.c_char_p, dp])
    _declare(host, "mhh_server_run", I, [P, I])
    _declare(host, "mhh_server_job_times", I, [P, I, dp, dp, dp])
    _declare(host, "mhh_server_get_result", I, [P, I, ctypes.c_char_p, dp])
    _declare(host, "mhh_server_peak_bytes", I, [P, dp])
    _declare(host, "mhh_server_progress", I, [P, dp, dp, I, ctypes.POINTER(I)])
    _declare(host, "mhh_server_destroy", I, [P])
    _declare(kern, "mhh_ctx_set_option", I, [P, ctypes.c_char_p, I])
    _declare(kern, "mhh_stats_profile", I, [P, P, dp, dp, S])
    _declare(kern, "mhh_ctx_scalar_offset", I, [P, dp])
    _declare(kern, "mhh_field_shift", I, [P, P, ctypes.c_double, S])
    _declare(kern, "mhh_ctx_device_bytes", I, [P, ctypes.POINTER(ctypes.c_size_t)])
    _declare(kern, "mhh_launch_count_add", I, [ctypes.c_longlong])
    _kern, _host = kern, host
    return kern, host


def check(rc, what="mhh"):
    if rc != 0:
        kern, host = load()
        # The message of the library whose entry point returned rc: each
        # keeps its last error until its next failure.
        fn = _last_call[0]
        if fn.startswith(("mhh_ensemble_", "mhh_server_")):
            msg = host.mhh_batch_last_error()
        elif fn.startswith("mhh_model_"):
            msg = host.mhh_model_last_error()
        else:
            msg = kern.mhh_last_error()
        msg = msg or b""
        raise MhhError(f"{what} failed ({rc}): {msg.decode(errors='replace')}", rc)


def set_option(name, value):
    """Process-wide kernel option of the native library (include/mhh.h)."""
    kern, _ = load()
    check(kern.mhh_set_option(name.encode(), int(value)), f"option {name}")


def launch_count():
    kern, _ = load()
    return int(kern.mhh_launch_count())


class Timing:
    """Live per-kernel-group CUDA-event timing of the native library."""

    @staticmethod
    def enable(on=True):
        kern, _ = load()
        check(kern.mhh_timing_enable(1 if on else 0))

    @staticmethod
    def reset():
        kern, _ = load()
        check(kern.mhh_timing_reset())

    @staticmethod
    def collect():
        """Returns {group: (launch groups, total ms)}."""
        kern, _ = load()
        check(kern.mhh_timing_collect())
        out = {}
        for q in range(kern.mhh_timing_count()):
            name, cnt, ms = ctypes.c_char_p(), ctypes.c_longlong(), ctypes.c_double()
            check(kern.mhh_timing_get(q, ctypes.byref(name), ctypes.byref(cnt), ctypes.byref(ms)))
            out[name.value.decode()] = (cnt.value, ms.value)
        return out


def _dptr(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class Model:
    """A device-resident model built from reference-style .ini text.

    ``Model(case)`` takes a cases.Case; ``Model(ini=..., z=...)`` raw input.
    """

    def __init__(self, case=None, precision=FP64, ini=None, z=None):
        kern, host = load()
        self.host = host
        self.kern = kern
        if case is not None:
            ini, z = case.to_ini(), case.z
        self._z = np.ascontiguousarray(z, dtype=np.float64)
        h = ctypes.c_void_p()
        check(host.mhh_model_create(ini.encode(), _dptr(self._z), len(self._z), precision, ctypes.byref(h)),
              "mhh_model_create")
        self.h = h
        self.precision = precision
        g = Grid()
        check(host.mhh_model_get_grid(self.h, ctypes.byref(g)))
        self.grid = g
        self.shape = (g.kcells, g.jcells, g.icells)
        if case is not None:
            for n in case.prognostic_names():
                self.set(n, case.embed(case.fields[n]))
            if case.swbuffer:
                for n, prof in case.buffer_profiles().items():
                    self.set_buffer_profile(n, prof)

    def close(self):
        if getattr(self, "h", None):
            self.host.mhh_model_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set(self, name, arr):
        a = np.ascontiguousarray(arr, dtype=np.float64).reshape(self.shape)
        check(self.host.mhh_model_set_field(self.h, name.encode(), _dptr(a)), f"set {name}")

    def set_buffer_profile(self, name, prof):
        p = np.ascontiguousarray(prof, dtype=np.float64)
        if p.size != self.grid.kcells:
            raise ValueError(f"buffer profile needs {self.grid.kcells} values")
        check(self.host.mhh_model_set_buffer_profile(self.h, name.encode(), _dptr(p)), f"buffer profile {name}")

    def get(self, name):
        a = np.empty(self.shape, dtype=np.float64)
        check(self.host.mhh_model_get_field(self.h, name.encode(), _dptr(a)), f"get {name}")
        return a

    def set_native(self, name, ptr):
        """Copies a host buffer in the model's precision (address ``ptr``)."""
        check(self.host.mhh_model_set_field_native(self.h, name.encode(), ctypes.c_void_p(ptr)), f"set {name}")

    def get_native(self, name, ptr):
        check(self.host.mhh_model_get_field_native(self.h, name.encode(), ctypes.c_void_p(ptr)), f"get {name}")

    def run_steps(self, n, fused=True):
        check(self.host.mhh_model_run_steps(self.h, n, 1 if fused else 0), "run_steps")

    def run_substeps(self, n, fused=True):
        check(self.host.mhh_model_run_substeps(self.h, n, 1 if fused else 0), "run_substeps")

    def _scalar(self, fn):
        v = ctypes.c_double()
        check(fn(self.h, ctypes.byref(v)))
        return v.value

    def cfl(self):
        return self._scalar(self.host.mhh_model_get_cfl)

    def dn(self):
        return self._scalar(self.host.mhh_model_get_dn)

    def div(self):
        return self._scalar(self.host.mhh_model_get_div)

    def dt(self):
        return self._scalar(self.host.mhh_model_get_dt)

    def time(self):
        return self._scalar(self.host.mhh_model_get_time)

    def profile(self, name):
        a = np.empty(self.grid.kcells, dtype=np.float64)
        check(self.host.mhh_model_get_profile(self.h, name.encode(), _dptr(a)))
        return a

    def surface(self, name):
        a = np.empty((self.grid.jcells, self.grid.icells), dtype=np.float64)
        check(self.host.mhh_model_get_surface(self.h, name.encode(), _dptr(a)))
        return a

    def set_stream(self, stream_handle):
        check(self.host.mhh_model_set_stream(self.h, ctypes.c_void_p(stream_handle)))

    def synchronize(self):
        check(self.host.mhh_model_synchronize(self.h))

    def save(self, directory):
        """Restart files of the current state in `directory`; returns iotime."""
        t = ctypes.c_int()
        check(self.host.mhh_model_save(self.h, os.fsencode(directory), ctypes.byref(t)), "save")
        return t.value

    def load(self, directory, iotime):
        check(self.host.mhh_model_load(self.h, os.fsencode(directory), int(iotime)), "load")

    def profile_stats(self, name):
        """Horizontal mean and variance of every level of field `name`
        (kcells values each), computed on the device in double."""
        self.synchronize()
        f, _ = self.device_fields()
        ptr = {"u": f.u, "v": f.v, "w": f.w, "th": f.s, "p": f.p, "evisc": f.evisc}[name]
        mean = np.empty(self.grid.kcells)
        var = np.empty(self.grid.kcells)
        check(self.kern.mhh_stats_profile(self.ctx(), ptr, _dptr(mean), _dptr(var), None), "stats_profile")
        if name == "th":
            mean += self.scalar_offset()
        return mean, var

    def scalar_offset(self):
        """The offset the scalar th is stored with on the device (thref0 in
        FP32 contexts with thermodynamics, else 0); host values are physical."""
        off = ctypes.c_double()
        check(self.kern.mhh_ctx_scalar_offset(self.ctx(), ctypes.byref(off)), "scalar_offset")
        return off.value

    def device_fields(self):
        f, b = Fields(), BcFields()
        check(self.host.mhh_model_get_device_fields(self.h, ctypes.byref(f), ctypes.byref(b)))
        return f, b

    def ctx(self):
        return self.host.mhh_model_get_ctx(self.h)


ENS_SEQUENTIAL, ENS_STREAMS, ENS_GRAPHS, ENS_BATCHED = 0, 1, 2, 3
SERVE_FIFO, SERVE_CONTINUOUS = 0, 1


class Ensemble:
    """Models of uneven sizes advanced together (include/mhh_batch.h).  The
    members stay owned by the caller and must outlive the ensemble."""

    def __init__(self, members=()):
        kern, host = load()
        self.host = host
        h = ctypes.c_void_p()
        check(host.mhh_ensemble_create(ctypes.byref(h)), "ensemble_create")
        self.h = h
        self.members = []
        for m in members:
            self.add(m)

    def add(self, model):
        check(self.host.mhh_ensemble_add(self.h, model.h), "ensemble_add")
        self.members.append(model)

    def autotune(self):
        buf = ctypes.create_string_buffer(4096)
        check(self.host.mhh_ensemble_autotune(self.h, buf, len(buf)), "ensemble_autotune")
        return buf.value.decode()

    def run_steps(self, n, mode=ENS_GRAPHS):
        check(self.host.mhh_ensemble_run_steps(self.h, n, mode), "ensemble_run_steps")

    def synchronize(self):
        check(self.host.mhh_ensemble_synchronize(self.h), "ensemble_synchronize")

    def close(self):
        if getattr(self, "h", None):
            self.host.mhh_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """Simulation jobs admitted by device-memory budget (include/mhh_batch.h)."""

    def __init__(self, budget_bytes, max_active):
        kern, host = load()
        self.host = host
        h = ctypes.c_void_p()
        check(host.mhh_server_create(float(budget_bytes), int(max_active), ctypes.byref(h)), "server_create")
        self.h = h
        self.cells = []

    def submit(self, case, nsteps, arrival=0.0, precision=FP32, keep=False):
        z = np.ascontiguousarray(case.z, dtype=np.float64)
        jid = ctypes.c_int()
        check(self.host.mhh_server_submit(self.h, case.to_ini().encode(), _dptr(z), len(z), precision, int(nsteps),
                                          float(arrival), 1 if keep else 0, ctypes.byref(jid)), "server_submit")
        for n in case.prognostic_names():
            a = np.ascontiguousarray(case.embed(case.fields[n]), dtype=np.float64)
            check(self.host.mhh_server_set_initial(self.h, jid.value, n.encode(), _dptr(a)), "server_set_initial")
        self.cells.append(case.itot * case.jtot * case.ktot * int(nsteps))
        return jid.value

    def run(self, mode=SERVE_CONTINUOUS):
        check(self.host.mhh_server_run(self.h, mode), "server_run")

    def times(self, job):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(self.host.mhh_server_job_times(self.h, job, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return a.value, b.value, c.value

    def result(self, job, name, shape):
        out = np.empty(shape, dtype=np.float64)
        check(self.host.mhh_server_get_result(self.h, job, name.encode(), _dptr(out)), "server_get_result")
        return out

    def progress(self):
        """(times, cells) of every completed step of the last run."""
        n = ctypes.c_int()
        check(self.host.mhh_server_progress(self.h, None, None, 0, ctypes.byref(n)))
        t = np.empty(n.value)
        c = np.empty(n.value)
        check(self.host.mhh_server_progress(self.h, _dptr(t), _dptr(c), n.value, ctypes.byref(n)))
        return t, c

    def peak_bytes(self):
        v = ctypes.c_double()
        check(self.host.mhh_server_peak_bytes(self.h, ctypes.byref(v)))
        return v.value

    def close(self):
        if getattr(self, "h", None):
            self.host.mhh_server_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

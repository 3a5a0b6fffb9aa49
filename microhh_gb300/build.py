"""In-tree build of the native libraries.

  lib/libmhh_gb300.so  -- the sm_103a CUDA kernels and the C-ABI (include/mhh.h)
  lib/libmhh_host.so   -- the C++ host layer with the reference's class API and
                          the mhh_model_* entry points (include/mhh_model.h)

Translation units compile in parallel with nvcc / g++ and are rebuilt only
when a source or header is newer than the library.
"""
import glob
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
INCLUDE = os.path.join(ROOT, "include")
CSRC = os.path.join(PKG, "csrc")
HOST = os.path.join(PKG, "host")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(ROOT, "_build")

LIB_KERNELS = os.path.join(LIBDIR, "libmhh_gb300.so")
LIB_HOST = os.path.join(LIBDIR, "libmhh_host.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _cudalib(cuda):
    for sub in ("lib64", os.path.join("targets", "sbsa-linux", "lib"), os.path.join("targets", "x86_64-linux", "lib")):
        d = os.path.join(cuda, sub)
        if os.path.isdir(d):
            return d
    return os.path.join(cuda, "lib64")


def _newest(paths):
    return max(os.path.getmtime(p) for p in paths)


def _run_parallel(cmds):
    procs = [(c, subprocess.Popen(c, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for c in cmds]
    failed = []
    for c, p in procs:
        out, _ = p.communicate()
        text = out.decode(errors="replace")
        text = "\n".join(l for l in text.splitlines() if "Warning: The 'compute_" not in l)
        if p.returncode != 0:
            failed.append((c, text))
        elif text.strip():
            sys.stderr.write(text + "\n")
    if failed:
        msg = "\n\n".join(" ".join(c) + "\n" + t for c, t in failed)
        raise RuntimeError("native build failed:\n" + msg)


def build(verbose=False, force=False, extra_nvcc=()):
    """Builds both libraries if needed; returns their paths."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)

    cu = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    hdr = sorted(glob.glob(os.path.join(CSRC, "*.cuh"))) + sorted(glob.glob(os.path.join(INCLUDE, "*.h")))
    if force or not os.path.exists(LIB_KERNELS) or _newest(cu + hdr) > os.path.getmtime(LIB_KERNELS):
        objs, cmds = [], []
        for src in cu:
            obj = os.path.join(OBJDIR, os.path.basename(src)[:-3] + ".o")
            objs.append(obj)
            cmds.append([nvcc, "-std=c++17", *ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                         "-I" + INCLUDE, "-I" + CSRC, *extra_nvcc, "-c", src, "-o", obj])
        _run_parallel(cmds)
        _run_parallel([[nvcc, *ARCH, "-shared", "-o", LIB_KERNELS, *objs, "-lcudart",
                        "-Xlinker", "-rpath," + _cudalib(cuda)]])

    hsrc = sorted(glob.glob(os.path.join(HOST, "*.cpp")))
    hhdr = sorted(glob.glob(os.path.join(HOST, "*.h"))) + sorted(glob.glob(os.path.join(INCLUDE, "*.h")))
    if force or not os.path.exists(LIB_HOST) or _newest(hsrc + hhdr + [LIB_KERNELS]) > os.path.getmtime(LIB_HOST):
        cxx = os.environ.get("CXX", "g++")
        cmds, objs = [], []
        for src in hsrc:
            obj = os.path.join(OBJDIR, os.path.basename(src)[:-4] + ".host.o")
            objs.append(obj)
            cmds.append([cxx, "-std=c++17", "-O2", "-fPIC", "-Wall", "-I" + INCLUDE,
                         "-I" + os.path.join(cuda, "include"), "-c", src, "-o", obj])
        _run_parallel(cmds)
        cudalib = _cudalib(cuda)
        _run_parallel([[cxx, "-shared", "-o", LIB_HOST, *objs, "-L" + LIBDIR, "-lmhh_gb300",
                        "-L" + cudalib, "-lcudart", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + cudalib]])
    return LIB_KERNELS, LIB_HOST


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))

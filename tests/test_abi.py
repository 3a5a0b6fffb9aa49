"""The C-ABI libraries build, load and export every declared entry point."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared(header):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(mhh_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def libs():
    from microhh_gb300 import build
    k, h = build.build()
    return ctypes.CDLL(k, mode=ctypes.RTLD_GLOBAL), ctypes.CDLL(h)


def test_kernel_library_exports_all(libs):
    kern, _ = libs
    names = declared("mhh.h")
    assert len(names) > 20
    missing = [n for n in names if not hasattr(kern, n)]
    assert not missing, missing


def test_host_library_exports_all(libs):
    _, host = libs
    names = declared("mhh_model.h") + declared("mhh_batch.h")
    missing = [n for n in names if not hasattr(host, n)]
    assert not missing, missing


def test_batch_errors_without_device(libs):
    """Argument errors of the ensemble and server entry points."""
    _, host = libs
    host.mhh_server_create.restype = ctypes.c_int
    host.mhh_server_create.argtypes = [ctypes.c_double, ctypes.c_int, ctypes.c_void_p]
    assert host.mhh_server_create(1e9, 0, None) == -1
    host.mhh_ensemble_add.restype = ctypes.c_int
    assert host.mhh_ensemble_add(None, None) == -1
    host.mhh_batch_last_error.restype = ctypes.c_char_p
    assert host.mhh_batch_last_error()


def test_errors_without_device(libs):
    """Argument errors come back as status codes, never as crashes."""
    kern, _ = libs
    kern.mhh_ctx_create.restype = ctypes.c_int
    assert kern.mhh_ctx_create(None, None, 64, None, None) == -1
    kern.mhh_last_error.restype = ctypes.c_char_p
    assert b"NULL" in kern.mhh_last_error()

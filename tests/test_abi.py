"""The C ABI library loads and exports every entry point of include/vfps.h
(no compute calls; runs without a GPU)."""
import ctypes as C
import os
import re

import pytest

from inovesa_gb300 import _lib
from inovesa_gb300.build import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not fn.endswith(".h"):
            continue
        with open(os.path.join(ROOT, "include", fn)) as f:
            text = f.read()
        names += re.findall(r"VFPS_API\s+[\w\s\*]+?\b(vfps_\w+)\s*\(", text)
    return names


@pytest.fixture(scope="module")
def lib():
    build()
    return _lib.lib()


def test_header_symbols_exported(lib):
    names = header_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_signatures_cover_header():
    names = set(header_functions())
    assert names == set(_lib.SIGNATURES), \
        names.symmetric_difference(set(_lib.SIGNATURES))


def test_null_arguments_are_rejected(lib):
    # invalid arguments are reported, not crashed on
    assert lib.vfps_create(None, 0) == _lib.VFPS_ERR_INVALID_ARGUMENT
    assert lib.vfps_ps_update_x_projection(None) == \
        _lib.VFPS_ERR_INVALID_ARGUMENT
    assert lib.vfps_map_apply(None) == _lib.VFPS_ERR_INVALID_ARGUMENT
    assert lib.vfps_batch_step(None, 1) == _lib.VFPS_ERR_INVALID_ARGUMENT
    msg = lib.vfps_last_error(None)
    assert msg and b"null" in msg


def test_create_reports_missing_device(lib):
    h = C.c_void_p()
    rc = lib.vfps_create(C.byref(h), 0)
    if rc == _lib.VFPS_OK:       # a GPU is present: nothing to check
        lib.vfps_destroy(h)
        return
    assert rc == _lib.VFPS_ERR_CUDA
    assert lib.vfps_last_error(None)
    rc = lib.vfps_create(C.byref(h), 999)
    assert rc in (_lib.VFPS_ERR_CUDA, _lib.VFPS_ERR_INVALID_ARGUMENT)

"""The C-ABI library builds for sm_103a, loads without a GPU and exports every symbol include/*.h declares."""
import ctypes
import os
import re

import pytest

import dpgsolver_gb300
from dpgsolver_gb300 import _lib

INCLUDE = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include")


def declared_functions():
    text = "".join(open(os.path.join(INCLUDE, h)).read() for h in sorted(os.listdir(INCLUDE)) if h.endswith(".h"))
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(dgpu_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def lib():
    dpgsolver_gb300.build()
    return ctypes.CDLL(_lib.LIB_PATH)


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("dgpu_create", "dgpu_compute_rhs", "dgpu_ssp_rk3_step", "dgpu_destroy"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared_functions()) <= set(_lib.EXPORTS)


def test_status_strings_without_gpu(lib):
    lib.dgpu_status_string.restype = ctypes.c_char_p
    assert lib.dgpu_status_string(0) == b"ok"
    assert lib.dgpu_status_string(1) == b"invalid argument"


def test_create_rejects_bad_arguments_without_gpu():
    l = dpgsolver_gb300.load()
    h = ctypes.c_void_p()
    st = l.dgpu_create(None, None, None, ctypes.byref(h))
    assert st == 1 and not h.value
    phys = _lib.Physics()
    phys.d = 4
    ops = _lib.TPOperators()
    mesh = _lib.Mesh()
    assert l.dgpu_create(ctypes.byref(phys), ctypes.byref(ops), ctypes.byref(mesh), ctypes.byref(h)) == 2
    assert b"d must be" in l.dgpu_last_error(None)

"""The C-ABI library builds for sm_103a, loads, and exports every symbol that
include/phantom_gb300.h declares (no compute calls: no GPU needed)."""
import ctypes
import os
import re

import pytest

from phantom_gb300 import build as B
from phantom_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "phantom_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ph_[a-z_0-9]+)\s*\(", src)))


@pytest.fixture(scope="module")
def libpath():
    if not os.path.exists(B.LIB):
        B.build()
    return B.LIB


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ("ph_init", "ph_build_tree", "ph_density", "ph_force", "ph_derivs", "ph_step"):
        assert s in syms


def test_library_exports_every_declared_symbol(libpath):
    L = ctypes.CDLL(libpath)
    missing = [s for s in declared_symbols() if not hasattr(L, s)]
    assert not missing, missing


def test_python_binding_covers_header():
    assert set(declared_symbols()) <= set(capi._SIGS)


def test_strerror_is_host_only(libpath):
    L = capi.lib(libpath)
    assert L.ph_strerror(7).decode() == "could not converge in density"
    assert L.ph_strerror(0).decode() == "ok"


def test_params_struct_layout():
    # ph_params: 10 int32, 22 doubles, int64, double, 4 int32 (include/phantom_gb300.h)
    assert ctypes.sizeof(capi.PhParams) == 10 * 4 + 22 * 8 + 8 + 8 + 4 * 4


def test_tune_struct_layout_and_host_checks(libpath):
    # ph_tune: 4 int32, 2 doubles, 1 int32 (include/phantom_gb300.h), padded to 8 B
    assert ctypes.sizeof(capi.PhTune) == 4 * 4 + 2 * 8 + 4 + 4
    L = capi.lib(libpath)
    t = capi.PhTune()
    assert L.ph_autotune(None, 0, ctypes.byref(t)) == 1  # PH_ERR_ARG without a context
    assert L.ph_get_tune(None, ctypes.byref(t)) == 1
    assert L.ph_set_tune(None, ctypes.byref(t)) == 1


def test_fortran_binding_covers_header():
    # every entry point of the header has an ISO_C_BINDING declaration in the
    # Fortran module a maintainer adds to the reference (include/ph_gpu_iface.F90)
    doc = open(os.path.join(ROOT, "include", "ph_gpu_iface.F90")).read()
    bound = set(re.findall(r'bind\(c,\s*name="(ph_[a-z_0-9]+)"\)', doc))
    missing = [s for s in declared_symbols() if s not in bound]
    assert not missing, missing

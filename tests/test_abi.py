"""The C-ABI library loads and exports every entry point the header declares (CPU)."""
import ctypes as C
import os
import re

import libmesh_gb300
from libmesh_gb300 import _capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    txt = open(os.path.join(ROOT, "include", "libmesh_gb300.h")).read()
    return sorted(set(re.findall(r"\blmg_status\s+(lmg_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared()
    assert "lmg_assemble" in names and "lmg_sparsity_build" in names and len(names) >= 20


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(_capi.LIB_PATH)
    for n in declared():
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    assert set(declared()) <= set(_capi.SIGNATURES)


def test_no_device_needed_for_host_entry_points():
    m = libmesh_gb300.Mesh.build_cube(1, 1, 1, libmesh_gb300.HEX8)
    assert m.n_elem == 1 and m.n_nodes == 8


def test_context_create_status():
    h = C.c_void_p()
    st = _capi.lib().lmg_context_create(C.byref(h), 0)
    if st == _capi.OK:  # a device is present
        assert _capi.lib().lmg_context_destroy(h) == _capi.OK
    else:               # no device: a clean status, no handle
        assert st == _capi.ERR_CUDA and not h.value

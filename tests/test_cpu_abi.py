"""The C-ABI library loads without a GPU and exports every entry point include/tfg.h declares."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from tfg import abi, lib, lib_path

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            names += re.findall(r"TFG_API\s+[^;(]*?\b(tfg_\w+)\s*\(", txt)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_symbols()
    assert "tfg_engine_create" in names and "tfg_step" in names and "tfg_potential_morse" in names
    assert len(names) >= 25


def test_library_exports_every_declared_symbol():
    L = C.CDLL(lib_path())
    missing = [n for n in declared_symbols() if not hasattr(L, n)]
    assert not missing, missing


def test_struct_layouts_match_header():
    # sizes implied by include/tfg.h on LP64
    assert C.sizeof(abi.Potential) == 4 + 4 + 16 + 4 + 4 + 4 + 4 + 8 + 12 + 4  # padded to 8
    assert C.sizeof(abi.Flux) == 36
    assert C.sizeof(abi.EngineDesc) == 88
    assert C.sizeof(abi.Reductions) == 8 * 7 + 8 * 8 + 16


def test_engine_create_without_device_reports_nodevice_or_rejects_bad_desc():
    L = lib()
    h = C.c_void_p()
    bad = abi.engine_desc((0, 0, 0), (10, 10, 10), (2, 2, 2), 1.0, 0.01)   # fewer than 3 cells
    rc = L.tfg_engine_create(C.byref(bad), C.byref(h))
    assert rc in (abi.TFG_E_INVAL, abi.TFG_E_NODEVICE)


def test_host_table_api_works_without_gpu():
    p = abi.P_POT()
    assert lib().tfg_potential_morse(1.0, 6.0, 0.0, 0.0001, 3.0, 0.001, 1, C.byref(p)) == 0
    e, f = C.c_float(), C.c_float()
    assert lib().tfg_potential_eval(p, 1.0, 1.0, 1.0, C.byref(e), C.byref(f)) == 1
    lib().tfg_potential_free(p)

"""The C-ABI library: it loads, and exports every function of include/*.h.

No device is touched: symbol lookup only.
"""

import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        text = re.sub(r"typedef[^;]*;", "", text, flags=re.S)
        text = re.sub(r"struct\s+\w+\s*\{.*?\};", "", text, flags=re.S)
        for m in re.finditer(r"([A-Za-z_]\w*)\s*\([^;{]*\)\s*;", text):
            names.add(m.group(1))
    return sorted(names)


def test_header_declares_hot_path():
    names = declared_functions()
    for fn in ("lb_collide", "lb_propagation", "lb_halo",
               "field_grad_compute", "field_halo", "phi_force_calculation",
               "phi_cahn_hilliard", "fe_symm_create", "ludwig_gb_binary_step"):
        assert fn in names


def test_library_exports_every_declared_function(gb):
    lib = ctypes.CDLL(gb.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_error_reporting_without_device(gb):
    """A call with invalid arguments fails with a message, no device use."""
    L = gb.lib()
    rc = L.cs_ntotal_set(None, (ctypes.c_int * 3)(4, 4, 4))
    assert rc == 1
    assert b"cs" in L.ludwig_gb_last_error()


def test_lattice_size_limit_without_device(gb):
    """Site indices are 32-bit unsigned: cs_init refuses 2^32 sites."""
    L = gb.lib()
    cs = ctypes.c_void_p()
    assert L.cs_create(None, ctypes.byref(cs)) == 0
    try:
        assert L.cs_ntotal_set(cs, (ctypes.c_int * 3)(2048, 2048, 1024)) == 0
        assert L.cs_init(cs) == 1
        assert b"2^32" in L.ludwig_gb_last_error()
    finally:
        L.cs_free(cs)
    cs = ctypes.c_void_p()
    assert L.cs_create(None, ctypes.byref(cs)) == 0
    try:
        assert L.cs_ntotal_set(cs, (ctypes.c_int * 3)(2048, 2048, 1023)) == 0
        assert L.cs_init(cs) == 0
    finally:
        L.cs_free(cs)

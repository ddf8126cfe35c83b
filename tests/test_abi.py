"""The C-ABI library: it loads, exports every function of include/*.h, and
its header's structures have the reference's layout.

No device is touched: symbol lookup, compilation and host-only calls.
"""

import ctypes
import glob
import json
import os
import re
import subprocess

import pytest

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


def _layout_tools():
    import sys
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_abi_layout
    return make_abi_layout


def test_structures_match_reference_layout():
    """Every structure a caller of the drop-in fills or reads (fe_t and its
    14-slot function table, the option and parameter structures) and every
    enumeration value, as include/ludwig_gb.h defines them, against what
    the reference's own headers give (tests/golden/abi_layout_reference.json,
    made by tests/golden/make_abi_layout.py)."""
    tools = _layout_tools()
    ours = tools.probe(["-I" + os.path.join(ROOT, "include")])
    with open(os.path.join(ROOT, "tests", "golden",
                           "abi_layout_reference.json")) as fh:
        ref = json.load(fh)
    assert sorted(ours) == sorted(ref)
    diff = {k: (ours[k], ref[k]) for k in ref if ours[k] != ref[k]}
    assert not diff, diff


def test_structures_match_reference_headers_live():
    """The same, compiled against the reference's headers themselves where
    its sources are present."""
    import oracle
    root = oracle.reference_root()
    if not root or not os.path.isdir(os.path.join(root, "src")):
        pytest.skip("reference sources not present")
    tools = _layout_tools()
    assert tools.probe(["-I" + os.path.join(ROOT, "include")]) == \
        tools.reference_layout(root)


def test_c_host_compiles_and_links(gb, tmp_path):
    """tests/c/ludwig_loop.c, a C host of the main loop, compiles against
    the header (its _Static_asserts pin the fe_t layout) and links against
    the library; running it needs a GPU (tests/test_c_host_gpu.py)."""
    libdir = os.path.dirname(gb.LIB_PATH)
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-Wall", "-Werror",
                    "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "ludwig_loop.c"),
                    "-L", libdir, "-lludwig_gb", "-lm",
                    "-Wl,-rpath," + libdir, "-o",
                    str(tmp_path / "ludwig_loop")], check=True)


def test_library_has_no_unresolved_own_symbols(gb):
    """Every function the library's objects call among themselves is
    defined in it (a C++ translation unit declaring a C function without C
    linkage would leave a mangled, unresolved name)."""
    out = subprocess.run(["nm", "-D", "--undefined-only", gb.LIB_PATH],
                         capture_output=True, text=True, check=True).stdout
    own = [ln for ln in out.splitlines()
           if "lgb" in ln or "ludwig_gb" in ln]
    assert not own, own


def test_cs_index_numbering_without_device(gb):
    """cs_index and cs_index_to_ijk follow src/coords.c:617-631 and
    :790-801 (halo-inclusive strides)."""
    L = gb.lib()
    cs = ctypes.c_void_p()
    assert L.cs_create(None, ctypes.byref(cs)) == 0
    try:
        assert L.cs_ntotal_set(cs, (ctypes.c_int * 3)(8, 6, 4)) == 0
        assert L.cs_nhalo_set(cs, 2) == 0
        assert L.cs_init(cs) == 0
        n = ctypes.c_int()
        assert L.cs_nsites(cs, ctypes.byref(n)) == 0
        assert n.value == 12 * 10 * 8
        xs, ys, zs = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        assert L.cs_strides(cs, ctypes.byref(xs), ctypes.byref(ys),
                            ctypes.byref(zs)) == 0
        assert (xs.value, ys.value, zs.value) == (80, 8, 1)
        c3 = (ctypes.c_int * 3)()
        for ic, jc, kc in ((1, 1, 1), (-1, 0, 6), (10, 8, -1), (3, 4, 2)):
            idx = L.cs_index(cs, ic, jc, kc)
            assert idx == 80 * (2 + ic - 1) + 8 * (2 + jc - 1) + (2 + kc - 1)
            assert L.cs_index_to_ijk(cs, idx, c3) == 0
            assert tuple(c3) == (ic, jc, kc)
    finally:
        L.cs_free(cs)


def test_physics_time_control_without_device(gb):
    """physics_control_* as src/physics.c:600-668: next_step advances the
    counter and stays positive while steps of the run remain; the time is
    t_start + t_current - 1."""
    L = gb.lib()
    ph = ctypes.c_void_p()
    assert L.physics_create(None, ctypes.byref(ph)) == 0
    try:
        assert L.physics_control_init_time(ph, 10, 3) == 0
        t = ctypes.c_double()
        left = [L.physics_control_next_step(ph) for _ in range(4)]
        assert left == [3, 2, 1, 0]
        assert L.physics_control_timestep(ph) == 14
        assert L.physics_control_time(ph, ctypes.byref(t)) == 0
        assert t.value == 10 + 14 - 1.0
        assert L.physics_e0_frequency_set(ph, 0.25) == 0
    finally:
        L.physics_free(ph)

"""The oracle against golden fixtures made by the reference itself.

tests/golden/make_golden.py ran the reference (built from its own sources)
on these inputs; the oracle must reproduce every value exactly.
"""

import hashlib
import os

import numpy as np
import pytest

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
A, B, KAPPA, MOB, ETA = -0.0625, 0.0625, 0.04, 0.3, 0.1


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def L_of(g):
    return tuple(int(v) for v in g["L"])


@pytest.mark.parametrize("name", ["run_8x6x4_s10", "run_12x10x8_s50",
                                  "run_map_10x8x6_s12"])
def test_oracle_run_matches_reference(orc, name):
    g = load(name)
    L = L_of(g)
    phi0 = orc.spinodal_init(L, int(g["seed"]), 0.0, 0.02)
    assert np.array_equal(phi0, g["phi0"])
    status = g["status"].reshape(-1).copy() if "status" in g else None
    st = orc.BinaryState(L, orc.lb_init_rest(L), phi0)
    orc.binary_steps(st, orc.symm_param(A, B, KAPPA), MOB,
                     orc.collide_param_m10(ETA), int(g["steps"]), status)
    for k in ("phi", "u", "rho", "force", "f"):
        if k in g:
            assert np.array_equal(getattr(st, k), g[k]), k


def test_oracle_1000_steps_matches_reference(orc):
    g = load("run_32cube_s1000")
    L = L_of(g)
    st = orc.BinaryState(L, orc.lb_init_rest(L), g["phi0"])
    orc.binary_steps(st, orc.symm_param(A, B, KAPPA), MOB,
                     orc.collide_param_m10(ETA), 1000)
    assert np.array_equal(st.phi, g["phi"])
    # f, u, rho and force are pinned by the SHA-256 of the reference's arrays
    for k in ("f", "u", "rho", "force"):
        a = np.ascontiguousarray(getattr(st, k), "<f8")
        assert hashlib.sha256(a.tobytes()).hexdigest() == str(g["sha256_" + k]), k


def test_oracle_collide(orc):
    g = load("collide_6x5x4")
    L = L_of(g)
    f, rho, u = orc.collide(L, orc.collide_param_m10(ETA), g["in_f"],
                            g["in_force"])
    assert np.array_equal(f, g["f"])
    assert np.array_equal(rho, g["rho"])
    assert np.array_equal(u, g["u"])


def test_oracle_propagate(orc):
    g = load("propagate_5x4x3")
    assert np.array_equal(orc.propagate(L_of(g), g["in_f"]), g["f"])


def test_oracle_grad(orc):
    g = load("grad_6x5x4")
    grad, delsq = orc.grad_7pt(L_of(g), g["in_phi"])
    assert np.array_equal(grad, g["grad"])
    assert np.array_equal(delsq, g["delsq"])


def test_oracle_force(orc):
    g = load("force_6x5x4")
    force = orc.phi_force(L_of(g), orc.symm_param(A, B, KAPPA), g["in_phi"])
    assert np.array_equal(force, g["force"])


def test_oracle_cahn_hilliard(orc):
    g = load("ch_6x5x4")
    phi = orc.cahn_hilliard(L_of(g), orc.symm_param(A, B, KAPPA), MOB,
                            g["in_phi"], g["in_u"])
    assert np.array_equal(phi, g["phi"])


def test_model_tables(orc):
    """Mode matrix properties (tests/unit/test_lb_model.c:272-377)."""
    cv, wv, ma, mi = orc.tables()
    assert np.allclose(ma @ mi, np.eye(19), atol=1e-14)
    assert abs(wv.sum() - 1.0) < 1e-15
    # orthogonality of modes under the weights
    gram = ma @ np.diag(wv) @ ma.T
    assert np.allclose(gram - np.diag(np.diag(gram)), 0, atol=1e-14)
    # opposite velocity exists for each p
    for p in range(19):
        assert any((cv[q] == -cv[p]).all() for q in range(19))


# --- cholesteric liquid crystal, blue phase I (A0 0.01, gamma 3, pitch 32) ---

GAMMA_ROT, ETA_LC = 0.5, 0.5


@pytest.mark.parametrize("name", ["lc_8x8x8_s3", "lc_16x12x8_s40"])
def test_oracle_lc_run_matches_reference(orc, name):
    g = load(name)
    L = L_of(g)
    p = orc.lc_param()
    assert np.array_equal(orc.lc_init_o8m(L, p), g["q0"])
    st = orc.LcState(L, orc.lb_init_rest(L), g["q0"])
    orc.lc_steps(st, p, GAMMA_ROT, orc.collide_param_m10(ETA_LC),
                 int(g["steps"]))
    for k in ("q", "u", "rho", "force", "f"):
        assert np.array_equal(getattr(st, k), g[k]), k


def test_oracle_lc_fields(orc):
    g = load("lc_fields_6x5x4")
    h, s, fed = orc.lc_fields(L_of(g), orc.lc_param(), g["in_q"])
    assert np.array_equal(h, g["h"])
    assert np.array_equal(s, g["stress"])
    assert np.array_equal(fed, g["fed"])


def test_oracle_beris_edwards(orc):
    g = load("lc_be_6x5x4")
    q = orc.lc_be_update(L_of(g), orc.lc_param(), GAMMA_ROT, g["in_q"],
                         g["in_u"])
    assert np.array_equal(q, g["q"])


# ---------------------------------------------------------------------------
# Two-distribution binary fluid (symmetric_lb, ndist = 2), mobility 0.45
# ---------------------------------------------------------------------------

@pytest.mark.parametrize("name", ["lb2_8x6x4_s10", "lb2_12x10x8_s60"])
def test_oracle_lb2_run_matches_reference(orc, name):
    g = load(name)
    L = L_of(g)
    phi0 = orc.spinodal_init(L, int(g["seed"]), 0.0, 0.02)
    st = orc.Lb2State(L, orc.lb_init_rest(L), orc.lb2_g_from_phi(phi0))
    orc.lb2_steps(st, orc.symm_param(A, B, KAPPA), 0.45,
                  orc.collide_param_m10(ETA), int(g["steps"]))
    for k in ("f", "g", "phi", "u"):
        assert np.array_equal(getattr(st, k), g[k]), k


def test_oracle_binary_collision_matches_reference(orc):
    g = load("collide2_6x5x4")
    f, gg, u = orc.collide_binary(L_of(g), orc.symm_param(A, B, KAPPA),
                                  orc.collide_param_m10(ETA), 0.45,
                                  g["in_f"], g["in_g"], g["in_phi"])
    assert np.array_equal(f, g["f"])
    assert np.array_equal(gg, g["g"])
    assert np.array_equal(u, g["u"])


@pytest.mark.parametrize("nf", [1, 5])
def test_oracle_grad27(orc, nf):
    g = load("grad27_nf%d_6x5x4" % nf)
    grad, delsq = orc.grad_27pt(L_of(g), g["in_phi"])
    assert np.array_equal(grad, g["grad"])
    assert np.array_equal(delsq, g["delsq"])


@pytest.mark.parametrize("name", ["run_adv2_8x6x4_s10", "run_adv3_12x10x8_s30",
                                  "run_adv2_g27_10x8x6_s12",
                                  "run_adv3_g27_8x8x8_s20"])
def test_oracle_advection_orders_match_reference(orc, name):
    """2nd/3rd-order advective fluxes (and the 27-point gradient) through
    the whole step."""
    import ctypes
    g = load(name)
    L = L_of(g)
    lib = orc.lib()
    lib.orc_advection_order_set.argtypes = [ctypes.c_int]
    lib.orc_gradient_stencil_set.argtypes = [ctypes.c_int]
    lib.orc_advection_order_set(int(g["order"]))
    lib.orc_gradient_stencil_set(int(g["grad"]) if "grad" in g else 7)
    try:
        st = orc.BinaryState(L, orc.lb_init_rest(L), g["phi0"])
        orc.binary_steps(st, orc.symm_param(A, B, KAPPA), MOB,
                         orc.collide_param_m10(ETA), int(g["steps"]))
        for k in ("phi", "u", "f"):
            assert np.array_equal(getattr(st, k), g[k]), k
    finally:
        lib.orc_advection_order_set(1)
        lib.orc_gradient_stencil_set(7)


IO_CASES = ["io_d1_phi_bin", "io_d2_phi_asc", "io_d1_q_asc", "io_d1_q_bin"]


@pytest.mark.parametrize("name", IO_CASES)
def test_oracle_snapshot_files_match_reference(orc, name):
    """Snapshot files of lb_io_write / field_io_write, byte for byte."""
    g = load(name)
    nf = int(g["nf"])
    fields = {"q" if nf == 5 else "phi": g["in_phi"]}
    if int(g["hydro"]):
        fields.update(rho=g["in_rho"], vel=g["in_u"])
    got = orc.snapshot_files(L_of(g), int(g["step"]), f=g["in_f"],
                             ndist=int(g["ndist"]), fields=fields,
                             fmt=str(g["fmt"]))
    names = [str(s) for s in g["files"]]
    assert sorted(got) == names
    for k, fn in enumerate(names):
        assert got[fn] == g["file%d" % k].tobytes(), fn


def _length_fields():
    import sys
    sys.path.insert(0, GOLDEN)
    from make_golden import length_fields
    return length_fields((128, 128, 128))


def test_oracle_length_matches_reference_program(orc):
    """util/length_from_sk.c itself (compiled against oracle/fftw_api) on
    128^3 fields: the oracle's faithful L agrees with the printed value to
    its 6 significant digits (the program sums in FP32, the oracle in
    FP64: 1e-5 relative covers both)."""
    g = load("length_from_sk_128cube")
    fields = _length_fields()
    fields["spinodal_s0"] = orc.spinodal_init((128, 128, 128), 8361235,
                                              0.0, 0.02)
    for name, phi in fields.items():
        a = np.ascontiguousarray(phi, "<f8")
        assert hashlib.sha256(a.tobytes()).hexdigest() == str(
            g["sha256_" + name]), name
        ref = float(g["L_" + name])
        got = orc.length_from_sk(phi, True)
        assert abs(got - ref) <= 1e-5 * ref, (name, got, ref)
        assert "%g" % got == str(g["printed_" + name]) or abs(
            got - ref) <= 5e-6 * ref, (name, got, ref)

"""Parity of the CUDA liquid-crystal path (FP64) with the oracle and with
golden fixtures made by the reference itself: every value exact."""

import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.mark.parametrize("name", ["lc_8x8x8_s3", "lc_16x12x8_s40"])
def test_lc_steps_match_reference_golden(gb, name):
    g = load(name)
    L = tuple(int(v) for v in g["L"])
    s = gb.LiquidCrystal(L)
    s.q.set(g["q0"])
    s.step_reference_order(int(g["steps"]))
    got = s.state()
    for k in ("q", "u", "rho", "force", "f"):
        assert np.array_equal(got[k], g[k]), (
            "%s: max |diff| %g" % (k, np.abs(got[k] - g[k]).max()))


def test_lc_o8m_init_matches_reference(gb):
    g = load("lc_8x8x8_s3")
    s = gb.LiquidCrystal((8, 8, 8))
    s.init_o8m()
    np.testing.assert_allclose(s.q.get(), g["q0"], rtol=0, atol=1e-15)


def test_lc_fields_match_reference_golden(gb):
    g = load("lc_fields_6x5x4")
    L = tuple(int(v) for v in g["L"])
    s = gb.LiquidCrystal(L)
    s.q.set(g["in_q"])
    s.dq.compute()
    s.pth.stress_compute(s.fe)
    assert np.array_equal(s.pth.get(), g["stress"])
    # H through the Beris-Edwards update without hydrodynamics
    s.be.update(s.fe, s.q, s.dq, None, s.map)
    assert np.array_equal(s.be.h(), g["h"])


def test_beris_edwards_matches_reference_golden(gb):
    g = load("lc_be_6x5x4")
    L = tuple(int(v) for v in g["L"])
    s = gb.LiquidCrystal(L)
    s.q.set(g["in_q"])
    s.hydro.set(u=g["in_u"])
    s.dq.compute()
    s.be.update(s.fe, s.q, s.dq, s.hydro, s.map)
    assert np.array_equal(s.q.get(), g["q"])


@pytest.mark.parametrize("L,n", [((12, 10, 8), 5), ((32, 32, 32), 20)])
def test_lc_steps_match_oracle(gb, orc, L, n):
    s = gb.LiquidCrystal(L)
    s.init_o8m()
    q0 = s.q.get()
    s.step_reference_order(n)
    st = orc.LcState(L, orc.lb_init_rest(L), q0)
    orc.lc_steps(st, orc.lc_param(), 0.5, orc.collide_param_m10(0.5), n)
    got = s.state()
    for k in ("q", "u", "rho", "f"):
        assert np.array_equal(got[k], getattr(st, k)), k


@pytest.mark.parametrize("L,n", [((12, 10, 8), 5), ((16, 12, 8), 40)])
def test_lc_fused_step_equals_reference_order(gb, L, n):
    """The two-kernel fused LC step gives the same bits as the per-function
    calls (which match the reference's golden runs)."""
    a = gb.LiquidCrystal(L)
    a.init_o8m()
    b = gb.LiquidCrystal(L)
    b.init_o8m()
    a.step_reference_order(n)
    b.step(n)
    sa, sb = a.state(), b.state()
    for k in ("q", "u", "rho", "f"):
        assert np.array_equal(sa[k], sb[k]), k


def test_lc_fused_golden(gb):
    g = load("lc_16x12x8_s40")
    L = tuple(int(v) for v in g["L"])
    s = gb.LiquidCrystal(L)
    s.q.set(g["q0"])
    s.step(int(g["steps"]))
    got = s.state()
    for k in ("q", "u", "rho", "f"):
        assert np.array_equal(got[k], g[k]), k


def test_lc_fp32_close_to_fp64(gb):
    L = (16, 16, 16)
    a = gb.LiquidCrystal(L)
    a.init_o8m()
    b = gb.LiquidCrystal(L, precision=1)
    b.init_o8m()
    a.step(200)
    b.step(200)
    qa, qb = a.state()["q"], b.state()["q"]
    assert np.abs(qa - qb).max() < 1e-5 * np.abs(qa).max() * 100


@pytest.mark.parametrize("solid,sites", [(False, 0), (True, 0), (False, 2)])
@pytest.mark.parametrize("precision", [1, 2])
def test_lc_fp32_one_step_close_to_fp64(gb, solid, sites, precision):
    """One reduced-precision step (float arithmetic; f stored as float or
    scaled half) against one FP64 step from the same perturbed blue phase
    with flow, with and without solid sites: the float path's
    reduced-operation H, stress and Beris-Edwards forms (any summation
    order) and its split kernels must agree with the reference-order FP64
    path to float rounding (half storage: to its 11-bit mantissa).  Both
    kernels of the float step with one site per thread and with two (packed
    FP32x2; all-fluid lattices only)."""
    gb.tune_sites(sites)
    try:
        _one_step_close(gb, solid, precision)
    finally:
        gb.tune_sites(0)


def _one_step_close(gb, solid, precision):
    L = (16, 12, 40)
    rng = np.random.default_rng(11)
    a = gb.LiquidCrystal(L, eta=0.5, gamma_rot=0.5, redshift=0.9,
                         epsilon=0.7, e0=(0.01, -0.02, 0.005))
    a.init_o8m()
    q = a.q.get() + 0.01 * rng.standard_normal((5,) + L)
    u = 0.01 * rng.standard_normal((3,) + L)
    b = gb.LiquidCrystal(L, eta=0.5, gamma_rot=0.5, redshift=0.9,
                         epsilon=0.7, e0=(0.01, -0.02, 0.005),
                         precision=precision)
    st = (rng.random(L) < 0.1).astype(np.uint8) if solid else None
    for s in (a, b):
        s.q.set(q)
        rho, _, force = s.hydro.get()
        s.hydro.set(rho=rho, u=u, force=force)
        if st is not None:
            s.map.set_status(st)
        s.step(1)
    sa, sb = a.state(), b.state()
    # f starts at rest, so the new u is the force (a divergence of the
    # stress, which loses digits to cancellation): a looser bound there
    tol_f = 2e-6 if precision == 1 else 2e-3
    for k, tol in (("q", 2e-6), ("f", tol_f), ("u", 1e-4)):
        scale = np.abs(sa[k]).max()
        err = np.abs(sa[k] - sb[k]).max()
        assert err < tol * scale, (k, err, scale)


@pytest.mark.parametrize("precision", [1, 2])
@pytest.mark.parametrize("L", [(16, 12, 40), (11, 9, 37), (8, 8, 64),
                               (3, 5, 7)])
def test_lc_collide_direct_matches_ring(gb, L, precision):
    """The float LC force + collision kernel that reads the stress
    neighbours through L1 (the default on all-fluid lattices) against the
    one that streams stress planes through a shared-memory ring (asked for
    by tune_sites(1)): the same arithmetic on the same values."""
    out = {}
    for sites in (1, 0):
        gb.tune_sites(sites)
        try:
            s = gb.LiquidCrystal(L, eta=0.5, gamma_rot=0.5,
                                 precision=precision)
            s.init_o8m()
            s.step(10)
            out[sites] = s.state()
        finally:
            gb.tune_sites(0)
    for k in ("q", "u", "f", "rho"):
        scale = np.abs(out[1][k]).max()
        err = np.abs(out[0][k] - out[1][k]).max()
        assert err <= 1e-6 * scale, (k, err, scale)


@pytest.mark.parametrize("sites", [0, 1, 2])
def test_lc_fp32_ragged_lattice_close_to_fp64(gb, sites):
    """The float LC kernels on extents that are no multiple of the tile or
    of 4 (P planes copied element by element; with two sites a thread, an
    odd number of rows leaves the last thread one site)."""
    L = (11, 9, 37)
    a = gb.LiquidCrystal(L, eta=0.5, gamma_rot=0.5)
    b = gb.LiquidCrystal(L, eta=0.5, gamma_rot=0.5, precision=gb.FP32)
    gb.tune_sites(sites)
    try:
        for s in (a, b):
            s.init_o8m()
            s.step(20)
    finally:
        gb.tune_sites(0)
    qa, qb = a.q.get(), b.q.get()
    assert np.abs(qa - qb).max() < 1e-5 * np.abs(qa).max()
    ua, ub = a.state()["u"], b.state()["u"]
    assert np.abs(ua - ub).max() < 1e-3 * np.abs(ua).max()


def test_lc_time_dependent_field(gb):
    """A time-dependent electric field (src/blue_phase.c:210-226): the phase
    coswt = cos(2 pi f t) at the physics object's time, taken before each
    step.  The fused step (which advances the step counter itself) equals
    the per-function calls with physics_control_next_step before each
    step, and both equal a static field whose phase is set by hand to
    cos(2 pi f t_n), t_n = t_start + n - 1 (src/physics.c:622-630)."""
    import math
    L, freq, nsteps = (12, 10, 8), 0.013, 6
    kw = dict(eta=0.5, gamma_rot=0.5, epsilon=0.7, e0=(0.01, -0.02, 0.005))
    lib = gb.lib()
    fused = gb.LiquidCrystal(L, **kw)
    calls = gb.LiquidCrystal(L, **kw)
    manual = gb.LiquidCrystal(L, **kw)
    for s in (fused, calls, manual):
        s.init_o8m()
        lib.physics_control_init_time(s.phys.ptr, 0, nsteps)
    for s in (fused, calls):
        lib.physics_e0_frequency_set(s.phys.ptr, freq)

    lib.ludwig_gb_physics_use(fused.phys.ptr)
    fused.step(nsteps)
    assert lib.physics_control_timestep(fused.phys.ptr) == nsteps

    lib.ludwig_gb_physics_use(calls.phys.ptr)
    for _ in range(nsteps):
        lib.physics_control_next_step(calls.phys.ptr)
        calls.step_reference_order(1)

    lib.ludwig_gb_physics_use(manual.phys.ptr)
    p = manual.fe.param
    for n in range(1, nsteps + 1):
        p.coswt = math.cos(2.0 * math.pi * freq * (0 + n - 1.0))
        gb._check(lib.fe_lc_param_set(manual.fe.ptr, ctypes.byref(p)),
                  "fe_lc_param_set")
        manual.step(1)

    a, b, c = fused.state(), calls.state(), manual.state()
    for k in ("q", "u", "rho", "f"):
        assert np.array_equal(a[k], b[k]), k
        assert np.array_equal(a[k], c[k]), k
    # and the field did act: a static field gives another trajectory
    static = gb.LiquidCrystal(L, **kw)
    static.init_o8m()
    lib.ludwig_gb_physics_use(static.phys.ptr)
    static.step(nsteps)
    assert not np.array_equal(static.q.get(), a["q"])

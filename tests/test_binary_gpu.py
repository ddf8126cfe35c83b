"""Parity of the CUDA binary-fluid path with the CPU oracle (FP64: exact).

The oracle is pinned bit for bit to the reference's own build
(tests/test_oracle_golden.py against the fixtures of tests/golden/).  Every FP64 comparison here is
exact equality of every value.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A, B, KAPPA, MOB, ETA = -0.0625, 0.0625, 0.04, 0.3, 0.1
SIZES = [(8, 6, 4), (5, 4, 3), (16, 16, 16), (33, 7, 40), (2, 2, 2)]


def rand_f(L, rng, amp=1e-3):
    """Distributions near rest equilibrium with random perturbations."""
    import oracle
    f = oracle.lb_init_rest(L)
    return f * (1.0 + amp * rng.standard_normal(f.shape))


@pytest.mark.parametrize("L", SIZES)
def test_propagation_exact(gb, orc, L):
    rng = np.random.default_rng(1)
    s = gb.BinaryFluid(L)
    f = rng.standard_normal((19,) + L)
    s.lb.set(f)
    s.lb.halo()
    s.lb.propagation()
    assert np.array_equal(s.lb.get(), orc.propagate(L, f))
    # two propagations in a row compose
    s.lb.propagation()
    assert np.array_equal(s.lb.get(), orc.propagate(L, orc.propagate(L, f)))


@pytest.mark.parametrize("L", SIZES)
def test_collide_exact(gb, orc, L):
    rng = np.random.default_rng(2)
    s = gb.BinaryFluid(L, eta=ETA)
    f = rand_f(L, rng)
    force = 1e-4 * rng.standard_normal((3,) + L)
    s.lb.set(f)
    s.hydro.set(force=force)
    s.lb.collide(s.hydro, s.map, s.fe)
    rho, u, _ = s.hydro.get()
    fo, ro, uo = orc.collide(L, orc.collide_param_m10(ETA), f, force)
    assert np.array_equal(s.lb.get(), fo)
    assert np.array_equal(rho, ro)
    assert np.array_equal(u, uo)


@pytest.mark.parametrize("L", SIZES)
def test_grad_exact(gb, orc, L):
    rng = np.random.default_rng(3)
    s = gb.BinaryFluid(L)
    phi = rng.uniform(-1, 1, (1,) + L)
    s.phi.set(phi)
    s.dphi.compute()
    g, d = s.dphi.get()
    go, do = orc.grad_7pt(L, phi)
    assert np.array_equal(g, go) and np.array_equal(d, do)


@pytest.mark.parametrize("L", SIZES)
def test_force_exact(gb, orc, L):
    rng = np.random.default_rng(4)
    s = gb.BinaryFluid(L)
    phi = rng.uniform(-1, 1, (1,) + L)
    s.phi.set(phi)
    s.hydro.f_zero()
    s.dphi.compute()
    gb.phi_force_calculation(s.pe, s.cs, s.pth, s.fe, s.map, s.phi, s.hydro)
    _, _, force = s.hydro.get()
    fe = orc.symm_param(A, B, KAPPA)
    assert np.array_equal(force, orc.phi_force(L, fe, phi))


@pytest.mark.parametrize("L", SIZES)
def test_cahn_hilliard_exact(gb, orc, L):
    rng = np.random.default_rng(5)
    s = gb.BinaryFluid(L, mobility=MOB)
    phi = rng.uniform(-1, 1, (1,) + L)
    u = 0.01 * rng.standard_normal((3,) + L)
    s.phi.set(phi)
    s.hydro.set(u=u)
    s.dphi.compute()
    gb.phi_cahn_hilliard(s.pch, s.fe, s.phi, s.hydro, s.map)
    fe = orc.symm_param(A, B, KAPPA)
    assert np.array_equal(s.phi.get(), orc.cahn_hilliard(L, fe, MOB, phi, u))


def oracle_run(orc, L, nsteps, seed=8361235, status=None):
    fe = orc.symm_param(A, B, KAPPA)
    cp = orc.collide_param_m10(ETA)
    st = orc.BinaryState(L, orc.lb_init_rest(L),
                         orc.spinodal_init(L, seed, 0.0, 0.02))
    orc.binary_steps(st, fe, MOB, cp, nsteps, status)
    return st


def assert_state_equal(got, st, force=False):
    for name in ("phi", "u", "rho", "f") + (("force",) if force else ()):
        ref = getattr(st, name)
        assert np.array_equal(got[name], ref), (
            "%s: max |diff| %g" % (name, np.abs(got[name] - ref).max()))


@pytest.mark.parametrize("L", [(8, 6, 4), (16, 16, 16)])
def test_reference_order_steps_exact(gb, orc, L):
    s = gb.BinaryFluid(L, mobility=MOB, eta=ETA)
    s.phi.init_spinodal(8361235, 0.0, 0.02)
    s.step_reference_order(10)
    assert_state_equal(s.state(), oracle_run(orc, L, 10), force=True)


@pytest.mark.parametrize("L,n", [((8, 6, 4), 10), ((5, 4, 3), 7),
                                 ((40, 24, 64), 21), ((33, 17, 35), 4)])
def test_fused_fp64_exact(gb, orc, L, n):
    s = gb.BinaryFluid(L, mobility=MOB, eta=ETA)
    s.phi.init_spinodal(8361235, 0.0, 0.02)
    s.step(n)
    assert_state_equal(s.state(), oracle_run(orc, L, n))


def test_fused_and_separate_calls_mix(gb, orc):
    L = (12, 10, 8)
    s = gb.BinaryFluid(L, mobility=MOB, eta=ETA)
    s.phi.init_spinodal(77, 0.0, 0.02)
    s.step(3)
    s.step_reference_order(2)
    s.step(5)
    assert_state_equal(s.state(), oracle_run(orc, L, 10, seed=77))


def test_fused_with_solid_sites_exact(gb, orc):
    L = (12, 10, 8)
    rng = np.random.default_rng(6)
    status = (rng.uniform(size=L) < 0.1).astype(np.uint8)
    s = gb.BinaryFluid(L, mobility=MOB, eta=ETA)
    s.map.set_status(status)
    s.phi.init_spinodal(8361235, 0.0, 0.02)
    s.step(6)
    st = oracle_run(orc, L, 6, status=status.reshape(-1).copy())
    got = s.state()
    fluid = status == 0
    for name in ("phi", "f"):
        assert np.array_equal(got[name], getattr(st, name)), name
    assert np.array_equal(got["u"], st.u)
    assert np.array_equal(got["rho"][0][fluid], st.rho[0][fluid])


def test_stats_match_oracle(gb, orc):
    L = (16, 12, 8)
    s = gb.BinaryFluid(L, mobility=MOB, eta=ETA)
    s.phi.init_spinodal(11, 0.0, 0.02)
    s.step(5)
    st = oracle_run(orc, L, 5, seed=11)
    got = s.phi.stats()
    ref = orc.field_stats(L, st.phi)
    assert abs(got[0] - ref[0]) <= 1e-16 * L[0] * L[1] * L[2]
    np.testing.assert_allclose(got[1:], ref[1:], rtol=1e-13, atol=1e-19)
    m = s.lb.moments()
    assert abs(m[0] - st.f.sum()) <= 1e-12
    fe = orc.symm_param(A, B, KAPPA)
    np.testing.assert_allclose(s.fe.fed_total(),
                               orc.symm_fed_total(L, fe, st.phi), rtol=1e-12)

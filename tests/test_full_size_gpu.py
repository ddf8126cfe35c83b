"""Parity at the benchmark's full sizes: the 256^3 binary fluid and the
128^3 cholesteric liquid crystal (blue phase I).

FP64: the fused steps against the oracle, every value bit for bit, for a
few steps at the full size (the oracle, OpenMP on the host cores, takes
seconds for them).  Reduced precision at 256^3, through properties that do
not depend on the size: total mass conserved to rounding (the rest
population is rebuilt from error-free sums), total phi conserved by the
flux form, total momentum of a fluid started at rest staying at rounding
level (the force is a divergence), and closeness to the FP64 path.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A, B, KAPPA, MOB, ETA = -0.0625, 0.0625, 0.04, 0.3, 0.1
N256 = (256, 256, 256)
N128 = (128, 128, 128)
SEED = 8361235


def test_fused_fp64_256cube_exact(gb, orc):
    st = orc.BinaryState(N256, orc.lb_init_rest(N256),
                         orc.spinodal_init(N256, SEED, 0.0, 0.02))
    orc.binary_steps(st, orc.symm_param(A, B, KAPPA), MOB,
                     orc.collide_param_m10(ETA), 3)
    s = gb.BinaryFluid(N256, mobility=MOB, eta=ETA)
    s.phi.init_spinodal(SEED, 0.0, 0.02)
    s.step(3)
    got = s.state()
    for name in ("phi", "u", "rho", "f"):
        assert np.array_equal(got[name], getattr(st, name)), name


@pytest.fixture(scope="module")
def fp64_256(gb):
    """FP64 (bit-exact) run at 256^3 after 200 steps: phi and the totals."""
    s = gb.BinaryFluid(N256, mobility=MOB, eta=ETA)
    s.phi.init_spinodal(SEED, 0.0, 0.02)
    s.step(200)
    u = s.hydro.get()[1]
    return s.phi.get(), np.abs(u).sum()


# Measured on a GB300 after 200 steps (mass drift, |momentum| / sum |u|,
# max |dphi|): FP32 0, 9e-11, 4.4e-9; FP16 1.9e-10, 3.9e-7, 4.8e-9.
@pytest.mark.parametrize("prec,dphi_tol,drift_tol,mom_tol", [
    (1, 1e-7, 1e-12, 1e-8),       # FP32-shifted
    (2, 1e-7, 1e-8, 1e-5),        # FP16 storage
])
def test_reduced_256cube_properties(gb, fp64_256, prec, dphi_tol,
                                    drift_tol, mom_tol):
    s = gb.BinaryFluid(N256, precision=prec, mobility=MOB, eta=ETA)
    s.phi.init_spinodal(SEED, 0.0, 0.02)
    phi0 = s.phi.get()
    m0 = s.lb.moments()[0]
    s.step(200)
    mom = s.lb.moments()
    phi = s.phi.get()
    phi64, usum64 = fp64_256
    print("prec %d: mass drift %.3g, momentum %s (sum |u| %.3g), "
          "max |dphi| %.3g" % (prec, (mom[0] - m0) / m0, mom[1:4], usum64,
                               np.abs(phi - phi64).max()))
    # mass: relative drift
    assert abs(mom[0] - m0) / m0 < drift_tol, (mom[0], m0)
    # momentum: zero at rest, the force sums to zero over the lattice
    assert np.abs(np.asarray(mom[1:4])).max() < mom_tol * usum64
    # total phi: conserved by the flux form up to the rounding of each
    # site's update (float: ~ulp(phi) per site, random signs)
    assert abs(phi.sum(dtype=np.float64) - phi0.sum(dtype=np.float64)) \
        < 1e-6 * np.abs(phi0).sum()
    # the trajectory follows the FP64 one
    assert np.abs(phi - phi64).max() < dphi_tol


def test_lc_fp64_128cube_exact(gb, orc):
    s = gb.LiquidCrystal(N128)
    s.init_o8m()
    q0 = s.q.get()
    s.step(2)
    st = orc.LcState(N128, orc.lb_init_rest(N128), q0)
    orc.lc_steps(st, orc.lc_param(), 0.5, orc.collide_param_m10(0.5), 2)
    got = s.state()
    for k in ("q", "u", "rho", "f"):
        assert np.array_equal(got[k], getattr(st, k)), k


def test_lc_fp32_128cube_close_to_fp64(gb):
    a = gb.LiquidCrystal(N128)
    b = gb.LiquidCrystal(N128, precision=1)
    for s in (a, b):
        s.init_o8m()
        s.step(20)
    sa, sb = a.state(), b.state()
    for k, tol in (("q", 1e-5), ("u", 1e-3)):
        scale = np.abs(sa[k]).max()
        err = np.abs(sa[k] - sb[k]).max()
        assert err < tol * scale, (k, err, scale)

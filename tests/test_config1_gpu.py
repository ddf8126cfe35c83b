"""Config 1 as specified, on the GPU: the FP64 symmetric binary fluid at 32^3
(M10, eta 0.1, A = -0.0625, B = 0.0625, kappa 0.04, M = 0.3, KISS99
spinodal start from seed 8361235) for 1000 steps, through the fused step and
through the per-function calls in the main-loop order of src/ludwig.c.

tests/golden/run_32cube_s1000.npz was written by the reference itself
(tests/golden/make_golden.py): phi after 1000 steps in full, and the SHA-256
of its f, u, rho and force arrays (little-endian doubles, C order), so that
the comparison is bit for bit on every field.  The tolerances the path is
specified with (1e-12 relative after 1000 steps; total mass and total phi
conserved to 1e-13 relative per step) are asserted as well.
"""

import hashlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
A, B, KAPPA, MOB, ETA = -0.0625, 0.0625, 0.04, 0.3, 0.1
CONSERVE_RTOL = 1e-13        # per step, total mass and total phi
FIELD_RTOL = 1e-12           # after 1000 steps


def sha256_of(a):
    return hashlib.sha256(np.ascontiguousarray(a, "<f8").tobytes()).hexdigest()


@pytest.fixture(scope="module")
def golden():
    return dict(np.load(os.path.join(GOLDEN, "run_32cube_s1000.npz")))


def system(gb, g):
    L = tuple(int(v) for v in g["L"])
    s = gb.BinaryFluid(L, a=A, b=B, kappa=KAPPA, mobility=MOB, eta=ETA)
    s.phi.init_spinodal(int(g["seed"]), 0.0, 0.02)
    assert np.array_equal(s.phi.get(), g["phi0"])
    return s


def check_against_golden(got, g, keys):
    phi = got["phi"]
    np.testing.assert_allclose(phi, g["phi"], rtol=FIELD_RTOL,
                               atol=FIELD_RTOL * np.abs(g["phi"]).max())
    assert np.array_equal(phi, g["phi"]), (
        "phi: max |diff| %g" % np.abs(phi - g["phi"]).max())
    for k in keys:
        assert sha256_of(got[k]) == str(g["sha256_" + k]), k


def totals(s):
    """(total mass, total phi) from the library's FP64 compensated sums."""
    return s.lb.moments()[0], s.phi.stats(0)[0]


def run_checking_conservation(s, nsteps, step):
    m0, p0 = totals(s)
    mprev, pprev = m0, p0
    worst = [0.0, 0.0]
    for _ in range(nsteps):
        step()
        m, p = totals(s)
        worst[0] = max(worst[0], abs(m - mprev) / abs(m0))
        # total phi starts near zero: relative to the sum of |phi|
        scale = float(np.abs(s.phi.get()).sum())
        worst[1] = max(worst[1], abs(p - pprev) / scale)
        mprev, pprev = m, p
    return worst


def test_config1_fused_1000_steps_bit_exact(gb, golden):
    s = system(gb, golden)
    s.step(1000)
    check_against_golden(s.state(), golden, ("f", "u", "rho"))


def test_config1_reference_order_1000_steps_bit_exact(gb, golden):
    s = system(gb, golden)
    s.step_reference_order(1000)
    check_against_golden(s.state(), golden, ("f", "u", "rho", "force"))


def test_config1_conservation_per_step(gb, golden):
    s = system(gb, golden)
    worst = run_checking_conservation(s, 1000, lambda: s.step(1))
    assert worst[0] <= CONSERVE_RTOL, "mass drift per step %g" % worst[0]
    assert worst[1] <= CONSERVE_RTOL, "phi drift per step %g" % worst[1]
    check_against_golden(s.state(), golden, ("f", "u", "rho"))

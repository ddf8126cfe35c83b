"""The float fused step with two sites per thread (packed FP32x2
arithmetic) against the one-site kernel and against itself under other
tilings.

The two forms run the same arithmetic with different instruction
sequences (the one-site kernel lets the compiler contract products and
sums; the packed form fuses a product with the sum that follows it), so
they agree to float rounding, not bit for bit.  Within the packed form a
site's values must not depend on the tiling: the halo ring of a tile is
computed one site at a time with the same roundings as a pair (sf1), so
every tile height and x chunk gives identical results.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MOB, ETA = 0.3, 0.1


def run(gb, L, prec, nsteps, sites, xchunk=0, ty=8, minb=0, seed=8361235):
    gb.tune_sites(sites)
    gb.tune(xchunk, ty, minb)
    try:
        s = gb.BinaryFluid(L, precision=prec, mobility=MOB, eta=ETA)
        s.phi.init_spinodal(seed, 0.0, 0.02)
        s.step(nsteps)
        return s.state()
    finally:
        gb.tune_sites(0)
        gb.tune(0, 8, 3)


@pytest.mark.parametrize("prec", [1, 2])
@pytest.mark.parametrize("L", [(24, 20, 16), (33, 17, 35), (16, 8, 64)])
def test_two_sites_match_one_site(gb, prec, L):
    one = run(gb, L, prec, 25, 1)
    two = run(gb, L, prec, 25, 2)
    tol = 2e-6 if prec == 1 else 2e-5
    assert np.abs(two["phi"] - one["phi"]).max() < tol
    assert np.abs(two["u"] - one["u"]).max() < tol
    np.testing.assert_allclose(two["f"], one["f"], rtol=0, atol=tol)
    # mass: the rest population is rebuilt from error-free sums in both
    assert abs(two["f"].sum() - one["f"].sum()) < 1e-9 * one["f"].sum()


@pytest.mark.parametrize("prec", [1, 2])
def test_two_sites_independent_of_tiling(gb, prec):
    L = (40, 27, 70)
    ref = run(gb, L, prec, 9, 2)
    for xchunk, ty, minb in ((8, 8, 2), (13, 16, 0), (64, 8, 4)):
        got = run(gb, L, prec, 9, 2, xchunk, ty, minb)
        for k in ("phi", "u", "rho", "f"):
            assert np.array_equal(got[k], ref[k]), (xchunk, ty, minb, k)


@pytest.mark.parametrize("L", [(16, 16, 32), (12, 10, 40), (12, 11, 40)])
def test_lc_two_site_kernels_match_one_site(gb, L):
    """The float LC step with both kernels two sites a thread (fields +
    Beris-Edwards, force + collision) against the one-site kernels: same
    arithmetic, float rounding apart (ny = 11: the last thread of each
    column has one site)."""
    out = {}
    for sites in (1, 2):
        gb.tune_sites(sites)
        try:
            s = gb.LiquidCrystal(L, precision=1)
            s.init_o8m()
            s.step(20)
            out[sites] = s.state()
        finally:
            gb.tune_sites(0)
    for k in ("q", "u", "rho", "f"):
        assert np.abs(out[2][k] - out[1][k]).max() < 1e-6, k

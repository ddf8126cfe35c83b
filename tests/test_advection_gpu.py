"""Second- and third-order advective fluxes (src/advection.c) through the
per-function FP64 step, with 7- and 27-point gradients, against runs of
the reference itself: exact.  The fused step refuses orders other than 1."""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("name", ["run_adv2_8x6x4_s10", "run_adv3_12x10x8_s30",
                                  "run_adv2_g27_10x8x6_s12",
                                  "run_adv3_g27_8x8x8_s20"])
def test_advection_orders_match_reference(gb, name):
    g = dict(np.load(os.path.join(GOLDEN, name + ".npz")))
    L = tuple(int(v) for v in g["L"])
    s = gb.BinaryFluid(L, gb.FP64, mobility=0.3, eta=0.1)
    if "grad" in g:
        s.dphi.set_stencil(int(g["grad"]))
    gb.advection_order(int(g["order"]))
    try:
        s.phi.set(g["phi0"])
        s.step_reference_order(int(g["steps"]))
        st = s.state()
        for k in ("phi", "u", "f"):
            assert np.array_equal(st[k], g[k]), (
                "%s: max |diff| %g" % (k, np.abs(st[k] - g[k]).max()))
    finally:
        gb.advection_order(1)


def test_fused_step_refuses_higher_orders(gb):
    s = gb.BinaryFluid((8, 8, 8), gb.FP64)
    gb.advection_order(2)
    try:
        with pytest.raises(gb.LudwigGBError):
            s.step(1)
    finally:
        gb.advection_order(1)

"""27-point gradient and Laplacian on the GPU (field_grad_compute with the
3d_27pt_fluid stencil) against fixtures from the reference itself: exact.
The fused steps use 7 points and refuse a 27-point gradient object."""

import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.mark.parametrize("nf", [1, 5])
def test_grad27_matches_reference(gb, nf):
    g = dict(np.load(os.path.join(GOLDEN, "grad27_nf%d_6x5x4.npz" % nf)))
    L = tuple(int(v) for v in g["L"])
    pe = gb.PE(0)
    cs = gb.Coords(pe, L)
    f = gb.Field(cs, nf, 2, gb.FP64, "f")
    fg = gb.FieldGrad(f, 2)
    fg.set_stencil(27)
    f.set(g["in_phi"])
    fg.compute()
    grad, delsq = fg.get()
    assert np.array_equal(grad, g["grad"])
    assert np.array_equal(delsq, g["delsq"])


def test_fused_step_refuses_27_points(gb):
    s = gb.BinaryFluid((8, 8, 8), gb.FP64)
    s.dphi.set_stencil(27)
    with pytest.raises(gb.LudwigGBError):
        s.step(1)

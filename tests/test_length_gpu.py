"""Domain length from the structure factor (util/length_from_sk.c), GPU
against the numpy restatement in the oracle, and against a known answer.

No reference output pins this metric (the reference's utility needs FFTW,
which is absent); the restatement follows its binning and quadrature,
including its wavevector quirk (faithful=True)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("faithful", [True, False])
@pytest.mark.parametrize("L", [(16, 16, 16), (32, 24, 20)])
def test_length_matches_oracle(gb, orc, L, faithful):
    rng = np.random.default_rng(7)
    pe = gb.PE(0)
    cs = gb.Coords(pe, L)
    phi = gb.Field(cs, 1)
    a = rng.uniform(-1, 1, (1,) + L)
    phi.set(a)
    length, sk, nk = phi.length_from_sk(faithful)
    sko, nko = orc.structure_factor(a, faithful)
    np.testing.assert_allclose(sk, sko, rtol=1e-10, atol=1e-9)
    assert np.array_equal(nk, nko)
    np.testing.assert_allclose(length, orc.length_from_sk(a, faithful),
                               rtol=1e-10)


def test_length_single_mode(gb):
    """cos(2 pi m x / N): all power at |k| = 2 pi m / N, so L is the
    wavelength N/m up to the half-bin offset of the quadrature."""
    N, m = 32, 4
    pe = gb.PE(0)
    cs = gb.Coords(pe, (N, N, N))
    phi = gb.Field(cs, 1)
    x = np.arange(N)
    a = np.cos(2 * np.pi * m * x / N)[:, None, None] * np.ones((N, N, N))
    phi.set(a[None])
    length, sk, nk = phi.length_from_sk(False)
    kbin = np.floor((2 * np.pi * m / N) * 128 / (np.sqrt(3) * np.pi))
    kc = (kbin + 0.5) * np.sqrt(3) * np.pi / 128
    assert abs(length - 2 * np.pi / kc) < 1e-9


def test_spinodal_length_grows(gb):
    """L(t) of the binary fluid grows during spinodal decomposition."""
    s = gb.BinaryFluid((32, 32, 32), mobility=0.3, eta=0.1)
    s.phi.init_spinodal(8361235, 0.0, 0.02)
    s.step(300)
    l1 = s.phi.length_from_sk()[0]
    s.step(700)
    l2 = s.phi.length_from_sk()[0]
    assert l2 > l1 > 0

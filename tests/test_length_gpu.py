"""Domain length from the structure factor (util/length_from_sk.c) on the
GPU: against the reference's own program and against the oracle.

tests/golden/length_from_sk_128cube.npz holds what the reference's
util/length_from_sk.c printed (compiled unmodified against the FFTW3
interface of oracle/fftw_api) for four 128^3 fields, with the SHA-256 of
each field; the fields are rebuilt here (the spinodal start, the FP64 run
of 600 steps from it, which is bit-exact with the reference's, and two
integer patterns) and checked against those digests first.  The program
prints 6 significant digits and sums in FP32, the library sums in FP64:
faithful = 1 must agree to 1e-5 relative.  Both modes are also checked
against the oracle's restatement (numpy FFT) to 1e-10."""

import hashlib
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
N128 = (128, 128, 128)


def sha256_of(a):
    return hashlib.sha256(np.ascontiguousarray(a, "<f8").tobytes()).hexdigest()


@pytest.fixture(scope="module")
def reference_lengths():
    return dict(np.load(os.path.join(GOLDEN, "length_from_sk_128cube.npz")))


def fields_128(gb):
    """The four fixture fields as library fields (FP64)."""
    sys.path.insert(0, GOLDEN)
    from make_golden import length_fields
    s = gb.BinaryFluid(N128, mobility=0.3, eta=0.1)
    s.phi.init_spinodal(8361235, 0.0, 0.02)
    out = {"spinodal_s0": s.phi.get()}
    s.step(600)
    out["spinodal_s600"] = s.phi.get()
    out.update(length_fields(N128))
    return s, out


def test_length_matches_reference_program(gb, orc, reference_lengths):
    g = reference_lengths
    s, fields = fields_128(gb)
    for name, phi in fields.items():
        assert sha256_of(phi) == str(g["sha256_" + name]), name
        s.phi.set(phi)
        ref = float(g["L_" + name])
        got, sk, nk = s.phi.length_from_sk(True)
        assert abs(got - ref) <= 1e-5 * ref, (name, got, ref)
        assert abs(np.sum(nk) - 128 * 128 * 65) == 0
        for faithful in (True, False):
            np.testing.assert_allclose(
                s.phi.length_from_sk(faithful)[0],
                orc.length_from_sk(phi, faithful), rtol=1e-10)


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

"""Reduced-precision forms against the FP64 oracle (32^3 spinodal, M = 0.3).

Tolerances are the measured GB300 errors with head-room:
  FP32-shifted after 1000 steps: max|dphi| 1.1e-6; mass drift below 1e-10
  (the rest population is rebuilt from error-free sums of the incoming
  and outgoing populations; 1.3e-12 after 1e4 steps at 256^3);
  FP16 storage: max|dphi| 1.3e-5, mass drift 3.5e-8.
The domain length L(t) of the reduced forms must be within 1% of FP64.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

A, B, KAPPA, MOB, ETA = -0.0625, 0.0625, 0.04, 0.3, 0.1
L3 = (32, 32, 32)
NSTEP = 1000


@pytest.fixture(scope="module")
def fp64_run(orc):
    st = orc.BinaryState(L3, orc.lb_init_rest(L3),
                         orc.spinodal_init(L3, 8361235, 0.0, 0.02))
    orc.binary_steps(st, orc.symm_param(A, B, KAPPA), MOB,
                     orc.collide_param_m10(ETA), NSTEP)
    return st


@pytest.mark.parametrize("prec,dphi_tol,drift_tol", [
    (1, 1e-5, 1e-10),       # FP32-shifted
    (2, 1e-4, 1e-6),        # FP16 storage
])
def test_reduced_precision_vs_fp64(gb, orc, fp64_run, prec, dphi_tol,
                                   drift_tol):
    s = gb.BinaryFluid(L3, precision=prec, mobility=MOB, eta=ETA)
    s.phi.init_spinodal(8361235, 0.0, 0.02)
    m0 = s.lb.moments()[0]
    s.step(NSTEP)
    m1 = s.lb.moments()[0]
    got = s.phi.get()
    assert np.abs(got - fp64_run.phi).max() < dphi_tol
    assert abs(m1 - m0) / m0 < drift_tol
    l64 = orc.length_from_sk(fp64_run.phi)
    lred = s.phi.length_from_sk()[0]
    assert abs(lred - l64) / l64 < 0.01
    # total phi is conserved by the flux form up to rounding
    assert abs(got.sum() - fp64_run.phi.sum()) < 1e-3


def test_fp32_state_roundtrip(gb):
    """Raw state out and back in leaves the trajectory unchanged."""
    L = (16, 12, 8)
    a = gb.BinaryFluid(L, precision=1, mobility=MOB, eta=ETA)
    a.phi.init_spinodal(5, 0.0, 0.02)
    a.step(7)
    pin = gb.PinnedState(a)
    lib = gb.lib()
    gb._check(lib.ludwig_gb_state_to_host_async(a.lb.ptr, a.phi.ptr,
                                                a.hydro.ptr, *pin.bufs[:3]),
              "to_host")
    gb.sync()
    ref = a.state()
    gb._check(lib.ludwig_gb_state_from_host_async(a.lb.ptr, a.phi.ptr,
                                                  a.hydro.ptr, *pin.bufs[:3]),
              "from_host")
    gb.sync()
    got = a.state()
    for k in ("f", "phi", "u"):
        assert np.array_equal(got[k], ref[k]), k


@pytest.mark.parametrize("L", [(17, 13, 37), (9, 24, 70)])
def test_fp32_ragged_lattice_close_to_fp64(gb, L):
    """Extents that are no multiple of the tile (8 x 32) or of 4: partial
    tiles, periodic halos wrapped element by element, short x-chunks."""
    a = gb.BinaryFluid(L, precision=gb.FP64, mobility=MOB, eta=ETA)
    b = gb.BinaryFluid(L, precision=gb.FP32, mobility=MOB, eta=ETA)
    for s in (a, b):
        s.phi.init_spinodal(77, 0.0, 0.02)
        s.step(40)
    assert np.abs(a.phi.get() - b.phi.get()).max() < 1e-6
    assert np.abs(a.lb.get() - b.lb.get()).max() < 1e-6


@pytest.mark.parametrize("prec,tol_phi,tol_f", [(1, 1e-6, 1e-6),
                                                (2, 1e-5, 1e-5)])
def test_reduced_with_solid_sites_close_to_fp64(gb, prec, tol_phi, tol_f):
    """The map branch of the reduced forms (no-flux faces next to solid
    sites, no collision on them) against the FP64 path, which matches the
    oracle bit for bit with the same map; a ragged z extent."""
    L = (12, 10, 40)
    rng = np.random.default_rng(6)
    status = (rng.uniform(size=L) < 0.1).astype(np.uint8)
    a = gb.BinaryFluid(L, precision=gb.FP64, mobility=MOB, eta=ETA)
    b = gb.BinaryFluid(L, precision=prec, mobility=MOB, eta=ETA)
    for s in (a, b):
        s.map.set_status(status)
        s.phi.init_spinodal(8361235, 0.0, 0.02)
    phi0 = b.phi.get()
    for s in (a, b):
        s.step(50)
    pa, pb = a.phi.get(), b.phi.get()
    assert np.abs(pa - pb).max() < tol_phi
    assert np.abs(a.lb.get() - b.lb.get()).max() < tol_f
    # no flux through a face next to a solid site: total phi is kept
    assert abs(pb.sum() - phi0.sum()) < 1e-4
    # solid sites keep their phi
    solid = status == 1
    assert np.array_equal(pb[0][solid], phi0[0][solid])


def test_fp16_scale_derived_from_the_range(gb):
    """FP16 storage: the scale maps the largest stored deviation into
    [2^10, 2^11), is a power of two, is derived again by the stepping and
    on request, and requantising by it leaves the trajectory close to the
    FP32 one."""
    L = (24, 20, 16)
    s16 = gb.BinaryFluid(L, precision=2, mobility=MOB, eta=ETA)
    s32 = gb.BinaryFluid(L, precision=1, mobility=MOB, eta=ETA)
    for s in (s16, s32):
        s.phi.init_spinodal(8361235, 0.0, 0.02)
        s.step(300)                 # crosses one derivation at step 256
    sc = s16.lb.fp16_rescale()
    assert sc == 2.0 ** round(np.log2(sc))
    f = s16.lb.get()
    w = np.array([12, 1, 1, 2, 1, 1, 1, 2, 1, 2, 2, 1, 2, 1, 1, 1, 2, 1, 1],
                 dtype=float) / 36.0
    dev = np.abs(f - w[:, None, None, None]).max()
    # largest deviation into [2^10, 2^11), the scale between 1 and 2^24
    # (dev carries the rounding of w_p in double: relative 1e-9 slack)
    if sc < 2.0 ** 24:
        assert 2.0 ** 10 * (1 - 1e-9) <= dev * sc < 2.0 ** 11 * (1 + 1e-9)
    else:
        assert dev * sc < 2.0 ** 11 * (1 + 1e-9)
    assert s16.lb.fp16_rescale() == sc          # idempotent
    s16.step(100)
    s32.step(100)
    assert np.abs(s16.phi.get() - s32.phi.get()).max() < 1e-4
    # handing f over from the host derives the scale from its range
    s16.lb.set(f)
    assert s16.lb.fp16_rescale() == sc

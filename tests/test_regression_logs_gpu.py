"""The GPU FP64 path against the reference's own regression logs.

The statistics the reference printed for three of its regression runs
(tests/regression/d3q19-short/*.log, read as text into
tests/golden/regression_logs.json by tests/golden/make_golden.py) are
recomputed here from the same inputs through this library's reference-
order API:

* serial-spin-fd1: symmetric binary fluid, 64^3, 27-point gradients,
  finite-difference Cahn-Hilliard, 10 steps;
* serial-spin-lb1: the same fluid on the two-distribution route
  (symmetric_lb), 27-point gradients, 10 steps;
* serial-init-bp1: cholesteric blue phase I (O8M), 32^3, redshift 0.83,
  one step;
* serial-symm-dr1: a drop of radius 16 in the symmetric binary fluid,
  64^3, 27-point gradients, second-order advection, one step;
* serial-init-bp2: blue phase II (O2), 32^3, redshift 0.91, one step;
* serial-relx-bp1: blue phase I relaxing without hydrodynamics, 100 steps;
* serial-chol-fld: a uniform nematic in a static electric field, 16^3,
  second-order advection, 10 steps;
* serial-init-br1, serial-init-br2: blue phases I and II rotated by Euler
  angles (90, 0, 0) and (45, 45, 0), one step;
* serial-symm-pat: spinodal patches (2^3 cubes of +-1, 10 % of -1) in the
  symmetric binary fluid, 64^3, 27-point gradients, second-order
  advection, one step;
* serial-init-lcr: random uniaxial directors (amplitude 0.01), one step;
* serial-init-lcb: a cholesteric helix along x with a 2^3 box of random
  directors at its centre, one step;
* d3q19-io/iodrop-mpi1-io1 and -io3: a drop of radius 8 (32^3, 27-point
  gradients, second-order advection) run 20 steps straight, and run 10
  steps, written to snapshot files, read back and run 10 more.

Values are compared to the digits the log prints (8 significant digits
for most, 11 for the free energy); sums whose terms cancel (momentum,
variance of rho) to an absolute bound.
"""

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
with open(os.path.join(GOLDEN, "regression_logs.json")) as _f:
    LOGS = json.load(_f)


# D3Q19 velocities in the reference's order (src/lb_d3q19.c)
CV = np.array([[0, 0, 0], [1, 1, 0], [1, 0, 1], [1, 0, 0], [1, 0, -1],
               [1, -1, 0], [0, 1, 1], [0, 1, 0], [0, 1, -1], [0, 0, 1],
               [0, 0, -1], [0, -1, 1], [0, -1, 0], [0, -1, -1], [-1, 1, 0],
               [-1, 0, 1], [-1, 0, 0], [-1, 0, -1], [-1, -1, 0]])


def close(got, ref, rel):
    """Printed value ref (rounded to its digits) against got."""
    return abs(got - ref) <= rel * abs(ref) + 1e-300


def check_scalars(got, ref, nsites, rel=6e-8):
    """total, mean, variance, min, max.  A total (and mean) whose terms
    cancel is only defined to the summation order's rounding, about
    1e-16 N max|value|: that bound applies where it exceeds the printed
    digits."""
    names = ("total", "mean", "variance", "min", "max")
    vmax = max(abs(ref[3]), abs(ref[4]))
    for k in range(5):
        tol = rel * abs(ref[k])
        if k == 0:
            tol = max(tol, 1e-14 * nsites * vmax)
        if k == 1:
            tol = max(tol, 1e-14 * vmax)
        if k == 2:
            # the reference sums squares without compensation: the
            # variance of a near-uniform field is rounding noise
            tol = max(tol, 1e-12 * vmax * vmax)
        assert abs(got[k] - ref[k]) <= tol, (names[k], got[k], ref[k])


def check_fe_line(got, ref):
    """The "[fe]" line: step, f, v, f/v, f_bulk/v, f_grad/v, redshift,
    printed with 11 significant digits."""
    names = ("f", "v", "f/v", "f_bulk/v", "f_grad/v", "redshift")
    for k in range(6):
        assert close(got[k], ref[1 + k], 1e-9), (names[k], got[k], ref[1 + k])


def rho_stats(f):
    rho = f.sum(axis=0)
    return rho.sum(), rho.min(), rho.max()


def check_common(s, ref, u, f, mom):
    """Density, momentum and velocity lines.  The total momentum is a sum
    whose terms cancel: it is defined only to the summation order's
    rounding, which the recursive-summation bound (N - 1) u sum|rho u_a|
    (u = 2^-53) limits; the log prints the reference's order."""
    tot, rmin, rmax = rho_stats(f)
    n = f[0].size
    jabs = max(np.abs(np.tensordot(CV[:, a], f, axes=(0, 0))).sum()
               for a in range(3))
    mom_tol = max(1e-13, (n - 1) * 2.0 ** -53 * jabs)
    assert close(tot, ref["rho"][0], 1e-9)
    assert close(rmin, ref["rho"][3], 1e-10)
    assert close(rmax, ref["rho"][4], 1e-10)
    # stats_velocity_minmax starts the minimum at FLT_MAX and the maximum
    # at FLT_MIN (the smallest positive float), as the reference does
    umin, umax, _ = s.hydro.velocity_minmax(s.map)
    flt_min = float(np.finfo(np.float32).tiny)
    flt_max = float(np.finfo(np.float32).max)
    for a in range(3):
        assert abs(mom[1 + a] - ref["total"][a]) < mom_tol
        assert close(umin[a], ref["minimum"][a], 1e-7)
        assert close(umax[a], ref["maximum"][a], 1e-7)
        assert umin[a] == min(flt_max, u[a].min())
        assert umax[a] == max(flt_min, u[a].max())


def test_serial_spin_fd1(gb):
    ref = LOGS["serial-spin-fd1"]
    s = gb.BinaryFluid((64, 64, 64), gb.FP64, a=-0.00625, b=0.00625,
                       kappa=0.004, mobility=1.25, eta=0.00625)
    s.dphi.set_stencil(27)
    s.phi.init_spinodal(8361235, 0.0, 0.1)
    check_scalars(s.phi.stats(), ref[0]["phi"], 64 ** 3)
    s.step_reference_order(10)
    check_scalars(s.phi.stats(), ref[1]["phi"], 64 ** 3)
    # the binary logs print the free energy per site
    assert close(s.fe.fed_total() / 64 ** 3, ref[1]["fed"][1], 1e-9)
    _, u, _ = s.hydro.get()
    check_common(s, ref[1], u, s.lb.get(), s.lb.moments())


def test_serial_spin_lb1(gb):
    ref = LOGS["serial-spin-lb1"]
    s = gb.BinaryFluidLB((64, 64, 64), a=-0.00625, b=0.00625, kappa=0.004,
                         mobility=3.75, eta=0.00625)
    s.dphi.set_stencil(27)
    s.init_spinodal(8361235, 0.0, 0.1)
    check_scalars(s.phi.stats(), ref[0]["phi"], 64 ** 3)
    s.step_reference_order(10)
    # statistics from phi = sum g after the step, gradients of the step
    gb.lib().phi_lb_to_field(s.phi.ptr, s.lb.ptr)
    check_scalars(s.phi.stats(), ref[1]["phi"], 64 ** 3)
    assert close(s.fe.fed_total() / 64 ** 3, ref[1]["fed"][1], 1e-9)
    _, u, _ = s.hydro.get()
    check_common(s, ref[1], u, s.lb.get(), s.lb.moments())


def test_serial_init_bp1(gb):
    ref = LOGS["serial-init-bp1"]
    s = gb.LiquidCrystal((32, 32, 32), eta=1.666666666666, gamma_rot=0.1,
                         a0=0.014384711, gamma=3.1764706, kappa0=0.01,
                         kappa1=0.01, xi=0.7, redshift=0.83, amplitude=-0.2,
                         q0=0.27768018)
    s.init_o8m()
    tags = ("Qxx", "Qxy", "Qxz", "Qyy", "Qyz")
    for n, t in enumerate(tags):
        check_scalars(s.q.stats(n), ref[0][t], 32 ** 3)
    assert close(s.fe.fed_total(), ref[0]["fe"][1], 1e-9)
    check_fe_line(s.fe.stats_info(s.map), ref[0]["fe"])
    s.step_reference_order(1)
    for n, t in enumerate(tags):
        check_scalars(s.q.stats(n), ref[1][t], 32 ** 3)
    # after a step the reference's statistics use the gradients of the step
    assert close(s.fe.fed_total(recompute=False), ref[1]["fe"][1], 1e-9)
    check_fe_line(s.fe.stats_info(s.map, recompute=False), ref[1]["fe"])
    _, u, _ = s.hydro.get()
    check_common(s, ref[1], u, s.lb.get(), s.lb.moments())


def test_serial_symm_dr1(gb):
    ref = LOGS["serial-symm-dr1"]
    A, K = -0.00625, 0.004
    s = gb.BinaryFluid((64, 64, 64), gb.FP64, a=A, b=-A, kappa=K,
                       mobility=1.25, eta=0.00625)
    s.dphi.set_stencil(27)
    gb.advection_order(2)
    try:
        s.phi.init_drop(np.sqrt(-2.0 * K / A), 16.0, 1.0, False)
        check_scalars(s.phi.stats(), ref[0]["phi"], 64 ** 3)
        s.dphi.compute()
        assert close(s.fe.fed_total() / 64 ** 3, ref[0]["fed"][1], 1e-9)
        s.step_reference_order(1)
        check_scalars(s.phi.stats(), ref[1]["phi"], 64 ** 3)
        assert close(s.fe.fed_total() / 64 ** 3, ref[1]["fed"][1], 1e-9)
        _, u, _ = s.hydro.get()
        check_common(s, ref[1], u, s.lb.get(), s.lb.moments())
    finally:
        gb.advection_order(1)


def lc_stats(s, ref, nsites):
    tags = ("Qxx", "Qxy", "Qxz", "Qyy", "Qyz")
    for n, t in enumerate(tags):
        check_scalars(s.q.stats(n), ref[t], nsites)


def test_serial_init_bp2(gb):
    ref = LOGS["serial-init-bp2"]
    s = gb.LiquidCrystal((32, 32, 32), eta=1.666666666666, gamma_rot=0.1,
                         a0=0.0069, gamma=3.0, kappa0=0.02, kappa1=0.02,
                         xi=0.7, redshift=0.91, amplitude=0.3, q0=0.1963495)
    s.init_o2()
    lc_stats(s, ref[0], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map), ref[0]["fe"])
    s.step_reference_order(1)
    lc_stats(s, ref[1], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map, recompute=False), ref[1]["fe"])
    _, u, _ = s.hydro.get()
    check_common(s, ref[1], u, s.lb.get(), s.lb.moments())


def test_serial_relx_bp1(gb):
    """No hydrodynamics: Q relaxes by the molecular field alone."""
    ref = LOGS["serial-relx-bp1"]
    s = gb.LiquidCrystal((32, 32, 32), gamma_rot=0.1, hydrodynamics=False,
                         a0=0.014384711, gamma=3.1764706, kappa0=0.01,
                         kappa1=0.01, xi=0.7, redshift=0.83, amplitude=-0.2,
                         q0=0.27768018)
    s.init_o8m()
    lc_stats(s, ref[0], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map), ref[0]["fe"])
    s.step_reference_order(100)
    lc_stats(s, ref[1], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map, recompute=False), ref[1]["fe"])


def test_serial_chol_fld(gb):
    """Uniform nematic along (1,1,0) in a static field e0 = (0.01, 0, 0)
    with dielectric anisotropy 41.4."""
    ref = LOGS["serial-chol-fld"]
    s = gb.LiquidCrystal((16, 16, 16), eta=0.135, eta_bulk=0.135,
                         gamma_rot=0.3, a0=0.084334998544,
                         gamma=3.085714285714, q0=0.0, kappa0=0.01,
                         kappa1=0.01, xi=0.7, redshift=1.0, amplitude=0.2,
                         epsilon=41.4, e0=(0.01, 0.0, 0.0))
    s.init_nematic((1.0, 1.0, 0.0))
    gb.advection_order(2)
    try:
        lc_stats(s, ref[0], 16 ** 3)
        # The reference prints the initial line before the field's phase
        # cos(wt) is first set (it is 0 until the first parameter commit),
        # so that f excludes the field term there: f/v = f_bulk/v + f_grad/v.
        got = s.fe.stats_info(s.map)
        assert close(got[3] + got[4], ref[0]["fe"][3], 1e-9)
        check_fe_line([got[3] * got[1], got[1], got[3] + got[4], got[3],
                       got[4], got[5]], ref[0]["fe"])
        s.step_reference_order(10)
        lc_stats(s, ref[1], 16 ** 3)
        check_fe_line(s.fe.stats_info(s.map, recompute=False), ref[1]["fe"])
        _, u, _ = s.hydro.get()
        check_common(s, ref[1], u, s.lb.get(), s.lb.moments())
    finally:
        gb.advection_order(1)


@pytest.mark.parametrize("name,init,angles,lc", [
    ("serial-init-br1", "o8m", (90.0, 0.0, 0.0),
     dict(a0=0.014384711, gamma=3.1764706, kappa0=0.01, kappa1=0.01,
          xi=0.7, redshift=0.83, amplitude=-0.2, q0=0.27768018)),
    ("serial-init-br2", "o2", (45.0, 45.0, 0.0),
     dict(a0=0.0069, gamma=3.0, kappa0=0.02, kappa1=0.02, xi=0.7,
          redshift=0.91, amplitude=0.3, q0=0.1963495)),
])
def test_serial_init_rotated(gb, name, init, angles, lc):
    ref = LOGS[name]
    s = gb.LiquidCrystal((32, 32, 32), eta=1.666666666666, gamma_rot=0.1,
                         **lc)
    getattr(s, "init_" + init)(angles)
    lc_stats(s, ref[0], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map), ref[0]["fe"])
    s.step_reference_order(1)
    lc_stats(s, ref[1], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map, recompute=False), ref[1]["fe"])
    _, u, _ = s.hydro.get()
    check_common(s, ref[1], u, s.lb.get(), s.lb.moments())


def test_serial_symm_pat(gb):
    ref = LOGS["serial-symm-pat"]
    s = gb.BinaryFluid((64, 64, 64), gb.FP64, a=-0.00625, b=0.00625,
                       kappa=0.004, mobility=1.25, eta=0.00625)
    s.dphi.set_stencil(27)
    gb.advection_order(2)
    try:
        s.phi.init_patches(8361235, 2, 0.1)
        check_scalars(s.phi.stats(), ref[0]["phi"], 64 ** 3)
        s.dphi.compute()
        assert close(s.fe.fed_total() / 64 ** 3, ref[0]["fed"][1], 1e-9)
        s.step_reference_order(1)
        check_scalars(s.phi.stats(), ref[1]["phi"], 64 ** 3)
        assert close(s.fe.fed_total() / 64 ** 3, ref[1]["fed"][1], 1e-9)
        _, u, _ = s.hydro.get()
        check_common(s, ref[1], u, s.lb.get(), s.lb.moments())
    finally:
        gb.advection_order(1)


def test_serial_init_lcr(gb):
    ref = LOGS["serial-init-lcr"]
    s = gb.LiquidCrystal((32, 32, 32), eta=0.1, gamma_rot=0.1,
                         a0=0.014384711, gamma=3.1764706, kappa0=0.01,
                         kappa1=0.01, xi=0.7, redshift=1.0, amplitude=0.01,
                         q0=0.27768018)
    s.init_random()
    lc_stats(s, ref[0], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map), ref[0]["fe"])
    s.step_reference_order(1)
    lc_stats(s, ref[1], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map, recompute=False), ref[1]["fe"])
    _, u, _ = s.hydro.get()
    check_common(s, ref[1], u, s.lb.get(), s.lb.moments())


def test_serial_init_lcb(gb):
    ref = LOGS["serial-init-lcb"]
    s = gb.LiquidCrystal((32, 32, 32), eta=0.1, gamma_rot=0.1,
                         a0=0.014384711, gamma=3.1764706, kappa0=0.01,
                         kappa1=0.01, xi=0.7, redshift=1.0, amplitude=0.01,
                         q0=0.27768018)
    s.init_cholesteric(0)
    s.random_rectangle((16, 16, 16), (17, 17, 17))
    lc_stats(s, ref[0], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map), ref[0]["fe"])
    s.step_reference_order(1)
    lc_stats(s, ref[1], 32 ** 3)
    check_fe_line(s.fe.stats_info(s.map, recompute=False), ref[1]["fe"])
    _, u, _ = s.hydro.get()
    check_common(s, ref[1], u, s.lb.get(), s.lb.moments())


def test_iodrop_restart(gb, tmp_path, monkeypatch):
    """The restart of d3q19-io/iodrop-mpi1-io3: 10 steps, snapshot files
    (distributions, phi, rho and velocity), a new system read from them,
    10 more steps; the statistics at step 20 are those of the
    uninterrupted run (-io1) and of the reference's own restart (-io3)."""
    io1, io3 = LOGS["iodrop-mpi1-io1"], LOGS["iodrop-mpi1-io3"]
    A, K, N = -0.00625, 0.004, 32 ** 3
    monkeypatch.chdir(tmp_path)
    gb.advection_order(2)
    try:
        def system():
            s = gb.BinaryFluid((32, 32, 32), gb.FP64, a=A, b=-A, kappa=K,
                               mobility=1.25, eta=0.00625)
            s.dphi.set_stencil(27)
            return s
        a = system()
        a.phi.init_drop(np.sqrt(-2.0 * K / A), 8.0, 1.0, False)
        check_scalars(a.phi.stats(), io1[0]["phi"], N)
        a.step_reference_order(10)
        check_scalars(a.phi.stats(), io1[1]["phi"], N)
        assert close(a.fe.fed_total() / N, io1[1]["fed"][1], 1e-9)
        a.lb.io_write(10)
        a.phi.io_write(10)
        a.hydro.io_write(10)
        b = system()
        b.lb.io_read(10)
        b.phi.io_read(10)
        b.hydro.io_read(10)
        check_scalars(b.phi.stats(), io3[0]["phi"], N)
        a.step_reference_order(10)
        b.step_reference_order(10)
        for s, ref in ((a, io1[2]), (b, io3[1])):
            check_scalars(s.phi.stats(), ref["phi"], N)
            assert close(s.fe.fed_total() / N, ref["fed"][1], 1e-9)
        assert np.array_equal(a.phi.get(), b.phi.get())
        assert np.array_equal(a.lb.get(), b.lb.get())
    finally:
        gb.advection_order(1)

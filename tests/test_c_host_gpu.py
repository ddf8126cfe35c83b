"""A C host compiled against include/ludwig_gb.h runs the reference's main
loop through the library (tests/c/ludwig_loop.c) and its results are
compared with the fixtures the reference itself made.

* binary: 8x6x4, 10 steps of the src/ludwig.c:528-860 call sequence from
  the KISS99 spinodal start; phi, f, u, rho and force bit for bit against
  tests/golden/run_8x6x4_s10.npz.  The reference's host layout (phi AOS,
  f SOA, every cs_index() site with periodic halo images) against the
  interior arrays.  fed, mu and the stress through fe->func at every
  cs_index() site, halo sites included: the total against
  stats_free_energy_symm, and every value against the same formula in
  numpy on the site's phi and gradients (same operation order: exact).
* lc: 8^3 blue phase I, 3 steps, Q handed over in the reference's AOS host
  layout; q, u, rho, force, f bit for bit against lc_8x8x8_s3.npz.
* lc_sites: fed, stress, htensor through fe->func against the reference's
  own values in lc_fields_6x5x4.npz; str_symm and str_anti against the
  reference's formulas (src/blue_phase.c:729-812) in numpy; the _v slots
  equal to the plain ones.
"""

import os
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLDEN = os.path.join(HERE, "golden")
NHALO = 2


def load(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


@pytest.fixture(scope="module")
def loop_exe(gb, tmp_path_factory):
    d = tmp_path_factory.mktemp("c_host")
    exe = str(d / "ludwig_loop")
    libdir = os.path.join(ROOT, "ludwig_gb300")
    subprocess.run(["gcc", "-std=gnu11", "-O2", "-Wall", "-Werror",
                    "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                    os.path.join(HERE, "c", "ludwig_loop.c"), "-L", libdir,
                    "-lludwig_gb", "-lm", "-Wl,-rpath," + libdir, "-o", exe],
                   check=True)
    return exe, d


def run(loop_exe, mode, *extra):
    exe, d = loop_exe
    prefix = str(d / mode)
    out = subprocess.run([exe, mode, prefix] + list(extra),
                         capture_output=True, text=True)
    assert out.returncode == 0, out.stderr
    return lambda name, shape: np.fromfile(
        "%s_%s.bin" % (prefix, name)).reshape(shape)


def halo_layout(a, model):
    """Interior (K, Lx, Ly, Lz) -> the reference's host layout of all
    cs_index() sites with periodic images in the halo."""
    K = a.shape[0]
    w = np.pad(a, ((0, 0),) + ((NHALO, NHALO),) * 3, mode="wrap")
    flat = w.reshape(K, -1)
    return flat.T.reshape(-1) if model == "aos" else flat.reshape(-1)


def test_binary_main_loop_from_c(loop_exe):
    g = load("run_8x6x4_s10")
    L = tuple(int(v) for v in g["L"])
    rd = run(loop_exe, "binary")
    for k, nc in (("phi", 1), ("f", 19), ("u", 3), ("rho", 1),
                  ("force", 3)):
        got = rd(k, (nc,) + L)
        assert np.array_equal(got, g[k]), k
    nall = tuple(n + 2 * NHALO for n in L)
    nsites = int(np.prod(nall))
    phi = rd("phi", (1,) + L)
    f = rd("f", (19,) + L)
    assert np.array_equal(rd("phi_cs_aos", (nsites,)),
                          halo_layout(phi, "aos"))
    assert np.array_equal(rd("f_cs_soa", (19 * nsites,)),
                          halo_layout(f, "soa"))

    fsum, total = rd("fed_total", (2,))
    np.testing.assert_allclose(fsum, total, rtol=1e-12)

    # per-site slots at every cs_index() site against numpy on the same
    # values (phi, gradients read back), in the slots' operation order
    a, b, kappa = -0.0625, 0.0625, 0.04
    grad = rd("grad", (3,) + L)
    dsq = rd("delsq", (1,) + L)[0]
    p = phi[0]
    g2 = grad[0] * grad[0] + grad[1] * grad[1] + grad[2] * grad[2]
    fed = (0.5 * a + 0.25 * b * p * p) * p * p + 0.5 * kappa * g2
    mu = a * p + b * p * p * p - kappa * dsq
    p0 = (0.5 * a * p * p + 0.75 * b * p * p * p * p - kappa * p * dsq
          - 0.5 * kappa * g2)
    st = np.zeros((9,) + L)
    for ia in range(3):
        for ib in range(3):
            st[3 * ia + ib] = p0 * float(ia == ib) + kappa * grad[ia] * grad[ib]
    assert np.array_equal(rd("fed_cs", (nsites,)),
                          halo_layout(fed[None], "aos"))
    assert np.array_equal(rd("mu_cs", (nsites,)),
                          halo_layout(mu[None], "aos"))
    assert np.array_equal(rd("stress_cs", (9 * nsites,)),
                          halo_layout(st, "aos"))
    assert np.array_equal(rd("stress_v_cs", (9 * nsites,)),
                          rd("stress_cs", (9 * nsites,)))


def test_lc_main_loop_from_c(loop_exe):
    g = load("lc_8x8x8_s3")
    L = tuple(int(v) for v in g["L"])
    exe, d = loop_exe
    qfile = str(d / "lc_q0_aos.bin")
    halo_layout(g["q0"], "aos").tofile(qfile)
    rd = run(loop_exe, "lc", qfile)
    for k, nc in (("q", 5), ("u", 3), ("rho", 1), ("force", 3), ("f", 19)):
        assert np.array_equal(rd(k, (nc,) + L), g[k]), k


def expand(t5):
    """(5, ...) -> (3, 3, ...) symmetric traceless, zz = 0 - xx - yy"""
    t = np.zeros((3, 3) + t5.shape[1:])
    t[0, 0], t[0, 1], t[0, 2] = t5[0], t5[1], t5[2]
    t[1, 0], t[1, 1], t[1, 2] = t5[1], t5[3], t5[4]
    t[2, 0], t[2, 1] = t5[2], t5[4]
    t[2, 2] = 0.0 - t5[0] - t5[3]
    return t


def test_lc_function_table_from_c(loop_exe):
    g = load("lc_fields_6x5x4")
    L = tuple(int(v) for v in g["L"])
    N = int(np.prod(L))
    exe, d = loop_exe
    qfile = str(d / "lc_sites_q_aos.bin")
    halo_layout(g["in_q"], "aos").tofile(qfile)
    rd = run(loop_exe, "lc_sites", qfile)

    def site_major(name):
        return rd(name, (N, 9)).T.reshape((3, 3) + L)

    assert np.array_equal(rd("fed", (1,) + L), g["fed"])
    stress = site_major("stress")
    assert np.array_equal(stress.reshape((9,) + L), g["stress"])
    h = site_major("htensor")
    h5 = np.array([h[0, 0], h[0, 1], h[0, 2], h[1, 1], h[1, 2]])
    assert np.array_equal(h5, g["h"])
    hh = expand(g["h"])
    q = expand(g["in_q"])
    anti = np.zeros((3, 3) + L)
    symm = stress.copy()
    for ia in range(3):
        for ib in range(3):
            for ic in range(3):
                anti[ia, ib] -= (q[ia, ic] * hh[ib, ic]
                                 - hh[ia, ic] * q[ib, ic])
                symm[ia, ib] += q[ia, ic] * hh[ib, ic] - hh[ia, ic] * q[ib, ic]
    assert np.array_equal(site_major("str_anti"), anti)
    assert np.array_equal(site_major("str_symm"), symm)
    for name in ("stress", "str_symm", "str_anti", "htensor"):
        assert np.array_equal(rd(name + "_v", (N, 9)), rd(name, (N, 9))), name

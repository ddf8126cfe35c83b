"""The oracle against the known answers the reference's own unit tests
hold for this path (values read from the reference's test sources).

* KISS99 draws: tests/unit/test_noise.c:95-125 (ns_uniform).
* Blue phase O8M structure, 64^3, 7-point gradients: Q, free-energy
  density, molecular field H and chiral stress at five sites,
  tests/unit/test_blue_phase.c:190-660 (tolerances as there: 1e-14 for
  Q, 1e-7 for the rest).
"""

import ctypes

import numpy as np
import pytest


def test_kiss99_known_draws(orc):
    L = orc.lib()
    L.orc_kiss_next.argtypes = [ctypes.POINTER(ctypes.c_uint)]
    L.orc_kiss_next.restype = ctypes.c_uint
    s = (ctypes.c_uint * 4)(0, 0, 0, 0)
    b = L.orc_kiss_next(s)
    assert list(s) == [1234567, 0, 0, 0] and b == 1234567
    s = (ctypes.c_uint * 4)(123, 456, 78, 9)
    b = L.orc_kiss_next(s)
    assert list(s) == [9730054, 1905505352, 2883582, 162000]
    assert b == 1915204894


# site (1-based, as the reference) -> expected values
Q = {
    (1, 1, 1): [0.0, -0.28284271247462, -0.28284271247462, 0.0,
                -0.28284271247462],
    (1, 1, 2): [0.2, 0.0, 0.0, -0.4, -0.48284271247462],
    (1, 1, 3): [0.0, 0.28284271247462, 0.28284271247462, 0.0,
                -0.28284271247462],
    (1, 12, 4): [-0.2, -0.08284271247462, 0.0, 0.4, 0.0],
    (2, 7, 6): [-0.2, 0.0, 0.0, -0.2, -0.08284271247462],
}
FED = {(1, 1, 1): 6.060508e-03, (1, 1, 2): 1.056203e-02,
       (1, 1, 3): 6.060508e-03, (1, 12, 4): 6.609012e-04,
       (2, 7, 6): 6.609012e-04}
H = {(1, 1, 1): [0.0, 0.0171194, 0.0171194, 0.0, 0.0171194],
     (1, 1, 2): [-0.0205178, 0.0, 0.0, 0.0303829, 0.0323891],
     (1, 1, 3): [0.0, -0.0171194, -0.0171194, 0.0, 0.0171194],
     (1, 12, 4): [0.0057295, 0.0023299, 0.0, -0.0111454, 0.0],
     (2, 7, 6): [0.0054159, 0.0, 0.0, 0.0057295, 0.0023299]}
S = {(1, 1, 1): [-7.887056e-03, -8.924220e-03, -9.837494e-03,
                 -9.837494e-03, -7.887056e-03, -8.924220e-03,
                 -8.924220e-03, -9.837494e-03, -7.887056e-03],
     (1, 1, 2): [7.375082e-03, 0.0, 0.0, 0.0, -4.179480e-02, -2.748179e-02,
                 0.0, -2.871796e-02, -5.329164e-03],
     (1, 1, 3): [-7.887056e-03, 8.924220e-03, 9.837494e-03, 9.837494e-03,
                 -7.887056e-03, -8.924220e-03, 8.924220e-03, -9.837494e-03,
                 -7.887056e-03],
     (1, 12, 4): [2.779621e-04, 7.180623e-04, 0.0, 1.308445e-03,
                  -5.056451e-03, 0.0, 0.0, 0.0, -1.007305e-04],
     (2, 7, 6): [-1.007305e-04, 0.0, 0.0, 0.0, 2.779621e-04, 7.180623e-04,
                 0.0, 1.308445e-03, -5.056451e-03]}


@pytest.fixture(scope="module")
def o8m(orc):
    L = (64, 64, 64)
    p = orc.lc_param(a0=0.014384711, gamma=3.1764706, kappa0=0.01,
                     kappa1=0.01, xi=0.7, amplitude=-0.2)
    p.q0 = np.sqrt(2.0) * 4.0 * np.arctan(1.0) * 1 * 16 / 64.0
    q = orc.lc_init_o8m(L, p)
    h, s, fed = orc.lc_fields(L, p, q)
    return q, h, s, fed


@pytest.mark.parametrize("site", sorted(Q))
def test_blue_phase_o8m_known_values(o8m, site):
    q, h, s, fed = o8m
    i, j, k = (c - 1 for c in site)
    assert np.abs(q[:, i, j, k] - Q[site]).max() < 1e-14
    assert abs(fed[0, i, j, k] - FED[site]) < 1e-7
    assert np.abs(h[:, i, j, k] - H[site]).max() < 1e-7
    assert np.abs(s[:, i, j, k] - S[site]).max() < 1e-7


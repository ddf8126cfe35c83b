"""The corrector network's CPU oracle (cnn_oracle.c) checked on its own.

The reference has no such network, so the oracle is pinned by central
finite differences of its loss and by the adjoint identities that tie the
three convolution forms together.  CPU only.
"""

import numpy as np
import pytest

N3 = (4, 4, 6)


def _params(orc, rng, small_last=False):
    p = np.zeros((orc.CNN_NLAYER, orc.CNN_PL), np.float32)
    for l in range(orc.CNN_NLAYER):
        cin = 5 if l == 0 else 32
        cout = 4 if l == orc.CNN_NLAYER - 1 else 32
        w = np.zeros((27, 32, 32), np.float32)
        w[:, :cout, :cin] = rng.uniform(-1, 1, (27, cout, cin)) * \
            np.sqrt(6.0 / (27 * cin))
        p[l, :orc.CNN_WL] = w.ravel()
        p[l, orc.CNN_WL:orc.CNN_WL + cout] = 0.1 * rng.standard_normal(cout)
    return p.ravel()


def _index(orc, l, t, n, c):
    return l * orc.CNN_PL + (t * 32 + n) * 32 + c


def test_gradient_matches_finite_differences(orc):
    rng = np.random.default_rng(1)
    N = N3[0] * N3[1] * N3[2]
    in5 = rng.standard_normal((5, N)).astype(np.float32)
    t4 = (0.1 * rng.standard_normal((4, N))).astype(np.float32)
    sc = np.ones(5, np.float32)
    p = _params(orc, rng)
    loss, g = orc.cnn_loss_grad(N3, in5, sc, t4, p, emulate=False)
    assert loss > 0
    idx = [_index(orc, 0, 3, 7, 2), _index(orc, 0, 26, 31, 4),
           _index(orc, 1, 13, 5, 17), _index(orc, 2, 0, 30, 31),
           _index(orc, 3, 20, 2, 9), _index(orc, 3, 5, 0, 0),
           1 * orc.CNN_PL + orc.CNN_WL + 3,      # a bias of layer 2
           3 * orc.CNN_PL + orc.CNN_WL + 1]      # a bias of the output
    for i in idx:
        p1, p2 = p.copy(), p.copy()
        p1[i] += np.float32(1e-3)
        p2[i] -= np.float32(1e-3)
        l1, _ = orc.cnn_loss_grad(N3, in5, sc, t4, p1, emulate=False)
        l2, _ = orc.cnn_loss_grad(N3, in5, sc, t4, p2, emulate=False)
        fd = (l1 - l2) / (float(p1[i]) - float(p2[i]))
        assert abs(g[i] - fd) <= 1e-5 * max(abs(fd), 1e-3), (i, g[i], fd)


def test_padding_channels_get_no_gradient(orc):
    rng = np.random.default_rng(2)
    N = N3[0] * N3[1] * N3[2]
    in5 = rng.standard_normal((5, N)).astype(np.float32)
    t4 = rng.standard_normal((4, N)).astype(np.float32)
    p = _params(orc, rng)
    _, g = orc.cnn_loss_grad(N3, in5, np.ones(5, np.float32), t4, p)
    g = g.reshape(orc.CNN_NLAYER, orc.CNN_PL)
    w0 = g[0, :orc.CNN_WL].reshape(27, 32, 32)
    w3 = g[3, :orc.CNN_WL].reshape(27, 32, 32)
    assert np.all(w0[:, :, 5:] == 0.0)           # layer-1 padding inputs
    assert np.all(w3[:, 4:, :] == 0.0)           # output padding
    assert np.all(g[3, orc.CNN_WL + 4:] == 0.0)


def test_conv_forms_are_adjoint(orc):
    """<conv(a), g> = <a, conv_T(g)> = <w, wgrad(g, a)> (no bias)."""
    rng = np.random.default_rng(3)
    n = (3, 5, 4)
    N = 60
    a = rng.standard_normal((N, 32))
    g = rng.standard_normal((N, 32))
    w = rng.standard_normal((27, 32, 32))
    z = orc.conv3_fwd(n, a, w, None)
    da = orc.conv3_bwd_data(n, g, w)
    dw, db = orc.conv3_wgrad(n, g, a)
    lhs = np.sum(z * g)
    assert np.isclose(lhs, np.sum(a * da), rtol=1e-12)
    assert np.isclose(lhs, np.sum(w * dw), rtol=1e-12)
    assert np.allclose(db, g.sum(axis=0), rtol=1e-12)


def test_conv_single_tap_is_a_shift(orc):
    """Only the tap (dx,dy,dz) = (1,0,-1) set: z(s) = a(s + e)."""
    n = (3, 4, 5)
    rng = np.random.default_rng(4)
    a = rng.standard_normal((60, 32))
    w = np.zeros((27, 32, 32))
    t = (1 + 1) * 9 + (0 + 1) * 3 + (-1 + 1)
    w[t] = np.eye(32)
    z = orc.conv3_fwd(n, a, w, None).reshape(3, 4, 5, 32)
    ar = a.reshape(3, 4, 5, 32)
    assert np.array_equal(z, np.roll(np.roll(ar, -1, axis=0), 1, axis=2))


def test_bf16_rounding(orc):
    v = np.array([1.0, 1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8, -3.14159, 0.0])
    r = orc.bf16_round(v)
    assert r[0] == 1.0
    assert r[1] == 1.0                       # tie -> even
    assert r[2] == 1.0 + 2.0 ** -6          # tie -> even (up)
    assert r[3] == -3.140625
    L = orc._cnn_lib()
    for x in v:
        assert L.orc_bf16_round(float(x)) == orc.bf16_round(np.array([x]))[0]


def test_emulated_precision_is_close(orc):
    rng = np.random.default_rng(5)
    N = N3[0] * N3[1] * N3[2]
    in5 = rng.standard_normal((5, N)).astype(np.float32)
    p = _params(orc, rng)
    sc = np.ones(5, np.float32)
    a = orc.cnn_forward(N3, in5, sc, p, emulate=False)
    b = orc.cnn_forward(N3, in5, sc, p, emulate=True)
    assert np.abs(a - b).max() < 0.05 * np.abs(a).max()

"""Tensor-core kernels of the learned corrector against the CPU oracle.

Single kernels (operands rounded to bf16, so the products are exact and
only the FP32 summation order differs): forward convolution, the
backward-data form (flipped, transposed weights) and the weight gradient,
on every tiling the kernels support and on grids where each CTA runs
several tiles.  Then the whole network (loss and gradients, oracle run
with the same bf16 rounding points), the Adam step, the fine -> coarse
restriction, and what the trained network gains on held-out seeds.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")


def dev(a):
    """A float32 CUDA tensor holding a, complete before the library (which
    runs on its own stream) reads it."""
    t = torch.from_numpy(np.ascontiguousarray(a, dtype=np.float32)).cuda()
    torch.cuda.synchronize()
    return t


def bf(orc, a):
    return orc.bf16_round(np.asarray(a)).astype(np.float32)


GEOMS = [(4, 4, 32), (2, 2, 64), (2, 2, 128), (2, 2, 256), (64, 32, 64)]


@pytest.mark.parametrize("n", GEOMS)
def test_conv3_forward(gb, orc, n):
    rng = np.random.default_rng(10)
    N = n[0] * n[1] * n[2]
    m = gb.Corrector(n)
    a = bf(orc, rng.standard_normal((N, 32)))
    w = bf(orc, 0.2 * rng.standard_normal((27, 32, 32)))
    b = rng.standard_normal(32).astype(np.float32)
    out = torch.empty((N, 32), dtype=torch.float32, device="cuda")
    da, dw, db = dev(a), dev(w), dev(b)      # keep the tensors alive
    m.conv3(da.data_ptr(), dw.data_ptr(), db.data_ptr(), 0, out.data_ptr())
    ref = orc.conv3_fwd(n, a, w, b)
    got = out.cpu().numpy().astype(np.float64)
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()


@pytest.mark.parametrize("n", [(2, 2, 128), (8, 40, 128), (3, 5, 256),
                               (160, 17, 128)])
@pytest.mark.parametrize("flip", [0, 1])
@pytest.mark.parametrize("mode", [1, 2, 3, 5])
def test_conv3_line_reuse_matches_per_tap(gb, orc, n, flip, mode):
    """nz a multiple of 128: the line-reuse kernel (runs of tiles along y,
    including runs of one tile and several runs per CTA) against the
    oracle, and bit for bit against the one-box-per-tap kernel; mode 3
    (three z taps per MMA, nz = 128; shifted partial sums added in the
    epilogue) to FP32 rounding of the per-tap kernel."""
    rng = np.random.default_rng(15)
    N = n[0] * n[1] * n[2]
    m = gb.Corrector(n)
    a = bf(orc, rng.standard_normal((N, 32)))
    w = bf(orc, 0.2 * rng.standard_normal((27, 32, 32)))
    b = rng.standard_normal(32).astype(np.float32)
    da, dw, db = dev(a), dev(w), dev(b)
    out_l = torch.empty((N, 32), dtype=torch.float32, device="cuda")
    out_t = torch.empty((N, 32), dtype=torch.float32, device="cuda")
    m.line_reuse(mode)
    m.conv3(da.data_ptr(), dw.data_ptr(), db.data_ptr(), flip,
            out_l.data_ptr())
    m.line_reuse(0)
    m.conv3(da.data_ptr(), dw.data_ptr(), db.data_ptr(), flip,
            out_t.data_ptr())
    got = out_l.cpu().numpy().astype(np.float64)
    if flip:
        ref = orc.conv3_bwd_data(n, a, w)
    else:
        ref = orc.conv3_fwd(n, a, w, b)
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()
    if mode in (3, 5) and n[2] == 128:
        # the same products summed in another order
        d = (out_l - out_t).abs().max().item()
        assert d <= 1e-5 * out_t.abs().max().item(), d
    else:
        # same products, same accumulation order: identical results
        assert torch.equal(out_l, out_t)


@pytest.mark.parametrize("n", [(4, 4, 32), (2, 2, 256), (64, 32, 64)])
def test_conv3_backward_data(gb, orc, n):
    rng = np.random.default_rng(11)
    N = n[0] * n[1] * n[2]
    m = gb.Corrector(n)
    g = bf(orc, rng.standard_normal((N, 32)))
    w = bf(orc, 0.2 * rng.standard_normal((27, 32, 32)))
    out = torch.empty((N, 32), dtype=torch.float32, device="cuda")
    dg, dw = dev(g), dev(w)
    m.conv3(dg.data_ptr(), dw.data_ptr(), 0, 1, out.data_ptr())
    ref = orc.conv3_bwd_data(n, g, w)
    got = out.cpu().numpy().astype(np.float64)
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max()


@pytest.mark.parametrize("n,line", [((4, 4, 32), 1), ((2, 4, 64), 1),
                                    ((2, 2, 256), 1), ((64, 32, 64), 1),
                                    ((2, 2, 256), 0), ((2, 2, 128), 1),
                                    ((8, 40, 128), 1), ((3, 17, 128), 1)])
def test_conv3_weight_gradient(gb, orc, n, line):
    """Per-tap kernel, and for nz a multiple of 128 the line-reuse kernel
    (gradient lines in a ring, the three dx lines of a (dy, dz) as one
    MMA's rows; runs of one to 16 tiles along y, several per CTA)."""
    rng = np.random.default_rng(12)
    N = n[0] * n[1] * n[2]
    m = gb.Corrector(n)
    m.line_reuse(line)
    g = bf(orc, rng.standard_normal((N, 32)))
    a = bf(orc, rng.standard_normal((N, 32)))
    dw = torch.empty((27, 32, 32), dtype=torch.float32, device="cuda")
    dg, da = dev(g), dev(a)
    m.wgrad3(dg.data_ptr(), da.data_ptr(), dw.data_ptr())
    ref, _ = orc.conv3_wgrad(n, g, a)
    got = dw.cpu().numpy().astype(np.float64)
    assert np.abs(got - ref).max() <= 2e-5 * np.abs(ref).max() * \
        max(1.0, np.sqrt(N / 4096.0))


def _data(rng, N):
    in5 = np.empty((5, N), np.float32)
    in5[0] = rng.uniform(-1, 1, N)
    in5[1:4] = 0.5 * rng.standard_normal((3, N))
    in5[4] = 1.0 + 0.1 * rng.standard_normal(N)
    t4 = (0.3 * rng.standard_normal((4, N))).astype(np.float32)
    return in5, t4


@pytest.mark.parametrize("n,mode", [((8, 8, 32), None), ((4, 4, 128), None),
                                    ((4, 4, 128), 3), ((4, 4, 128), 4),
                                    ((3, 17, 128), 4), ((3, 17, 128), 5)])
def test_network_loss_and_gradient_vs_oracle(gb, orc, n, mode):
    """The whole network (default form, or the given line form: 3 three z
    taps per MMA, 4 the same with the last layer's y taps folded into its
    MMAs) against the oracle with the same BF16 rounding points."""
    N = n[0] * n[1] * n[2]
    rng = np.random.default_rng(13)
    m = gb.Corrector(n, seed=7)
    if mode is not None:
        m.line_reuse(mode)
    one = np.ones(5, np.float32)
    m.set_scales(np.zeros(5), one, np.ones(4))
    # a trained-looking last layer: scale it up so every layer matters
    p = m.params()
    p[3 * 27680:3 * 27680 + 27648] *= 10.0
    m.set_params(p)
    in5, t4 = _data(rng, N)
    x, t = dev(in5), dev(t4)
    out = torch.empty((4, N), dtype=torch.float32, device="cuda")
    m.forward(x.data_ptr(), out.data_ptr())
    ref_out = orc.cnn_forward(n, in5, one, p, emulate=True)
    got = out.cpu().numpy()
    assert np.abs(got - ref_out).max() <= 1e-2 * np.abs(ref_out).max()

    loss = m.loss_grad(x.data_ptr(), t.data_ptr())
    ref_loss, ref_g = orc.cnn_loss_grad(n, in5, one, t4, p, emulate=True)
    assert abs(loss - ref_loss) <= 1e-3 * ref_loss
    g = m.grads().astype(np.float64).reshape(4, -1)
    rg = ref_g.reshape(4, -1)
    for l in range(4):
        rel = np.linalg.norm(g[l] - rg[l]) / np.linalg.norm(rg[l])
        assert rel < 2e-2, (l, rel)


def test_adam_step_and_training_reduces_loss(gb, orc):
    n = (8, 8, 32)
    N = 2048
    rng = np.random.default_rng(14)
    m = gb.Corrector(n, seed=3)
    m.set_scales(np.zeros(5), np.ones(5), np.ones(4))
    in5, t4 = _data(rng, N)
    # a learnable target: a smooth function of the inputs
    t4[0] = 0.5 * in5[0] - 0.2 * in5[1]
    t4[1:] = 0.1 * in5[2:5] - 0.1
    x, t = dev(in5), dev(t4)
    p0 = m.params().astype(np.float64)
    m.loss_grad(x.data_ptr(), t.data_ptr())
    g0 = m.grads().astype(np.float64)
    lr = 1e-3
    l0 = m.train_step(x.data_ptr(), t.data_ptr(), lr)
    p1 = m.params().astype(np.float64)
    # first Adam step: m_hat = g, v_hat = g^2 -> dp = -lr g / (|g| + eps)
    expect = p0 - lr * g0 / (np.abs(g0) + 1e-8)
    assert np.abs(p1 - expect).max() < 2e-6
    losses = [l0]
    for _ in range(60):
        losses.append(m.train_step(x.data_ptr(), t.data_ptr(), lr))
    assert losses[-1] < 0.3 * losses[0]


def test_restriction_matches_numpy(gb):
    fine = gb.BinaryFluid((16, 16, 16), gb.FP32, mobility=0.3, eta=0.1)
    fine.phi.init_spinodal(77, 0.0, 0.02)
    fine.step(301)
    from ludwig_gb300.corrector import coarse_params, FINE_PARAMS
    coarse = gb.BinaryFluid((8, 8, 8), gb.FP32, **coarse_params(FINE_PARAMS))
    gb.coarse_restrict(fine, coarse)
    f = fine.lb.get()
    phi = fine.phi.get()[0]
    _, u, _ = fine.hydro.get()
    cv = np.array(gb.CV if hasattr(gb, "CV") else [
        [0, 0, 0], [1, 1, 0], [1, 0, 1], [1, 0, 0], [1, 0, -1], [1, -1, 0],
        [0, 1, 1], [0, 1, 0], [0, 1, -1], [0, 0, 1], [0, 0, -1], [0, -1, 1],
        [0, -1, 0], [0, -1, -1], [-1, 1, 0], [-1, 0, 1], [-1, 0, 0],
        [-1, 0, -1], [-1, -1, 0]], dtype=np.float64)
    w = np.array([12, 1, 1, 2, 1, 1, 1, 2, 1, 2, 2, 1, 2, 1, 1, 1, 2, 1, 1]) / 36.0

    def blk(a):
        return a.reshape(8, 2, 8, 2, 8, 2).mean(axis=(1, 3, 5))

    rho = blk(f.sum(axis=0))
    j = np.stack([blk(np.tensordot(cv[:, a], f, 1)) for a in range(3)])
    pi = np.stack([[blk(np.tensordot(cv[:, a] * cv[:, b], f, 1))
                    for b in range(3)] for a in range(3)])
    eye = np.eye(3)[:, :, None, None, None]
    pneq = pi - eye * rho / 3.0 - j[:, None] * j[None, :] / rho
    jc = 2.0 * j
    pdev = jc[:, None] * jc[None, :] / rho + 4.0 * pneq
    fc = np.empty((19, 8, 8, 8))
    for p in range(19):
        q = np.outer(cv[p], cv[p]) - np.eye(3) / 3.0
        fc[p] = w[p] * (rho + 3.0 * np.tensordot(cv[p], jc, 1)
                        + 4.5 * np.einsum("ab,ab...->...", q, pdev))
    assert np.abs(coarse.lb.get() - fc).max() < 2e-6
    assert np.abs(coarse.phi.get()[0] - blk(phi)).max() < 1e-6
    rc, uc, _ = coarse.hydro.get()
    assert np.abs(uc - 2.0 * np.stack([blk(u[a]) for a in range(3)])).max() \
        < 1e-7
    assert np.abs(rc[0] - rho).max() < 1e-6
    # conservation: coarse totals are fine totals / 8
    assert abs(coarse.lb.moments()[0] - fine.lb.moments()[0] / 8) < 1e-3


@pytest.fixture(scope="module")
def trained(gb):
    from ludwig_gb300 import corrector as cr
    nfine = (64, 64, 64)
    X, Y = cr.make_pairs(nfine, [11, 12, 13, 14, 15, 16], 800, 100, 6)
    off, isc, osc = cr.scales_from(X, Y)
    T = cr.targets(X, Y, osc)
    m = gb.Corrector((32, 32, 32), seed=12345)
    m.set_scales(off, isc, osc)
    hist = cr.train(m, X, T, epochs=15, lr=2e-3)
    Xh, Yh = cr.make_pairs(nfine, [21, 22], 800, 100, 6)
    Th = cr.targets(Xh, Yh, osc)
    return cr, m, hist, cr.one_step_errors(m, Xh, Th)


def test_training_converges(trained):
    cr, m, hist, _ = trained
    assert np.all(np.isfinite(hist))
    assert hist[-1] < 0.8 * hist[0]


def test_network_gains_on_held_out_seeds(trained):
    """One coarse step from held-out fine states: the corrected coarse
    step is closer to the restricted fine run than the plain one."""
    cr, m, hist, (plain, corrected) = trained
    assert corrected < 0.7 * plain, (plain, corrected)


def test_rollout_and_fallback(trained):
    cr, m, _, _ = trained
    recs = cr.rollout(m, (64, 64, 64), 21, 800, 40, 20)
    assert all(np.isfinite(r["err_corrected"]) for r in recs)
    method, worst = cr.choose_method(recs)
    assert method in ("coarse+corrector", "fine")
    assert (method == "fine") == (worst > 0.02)


def test_rollout_pairs(trained, gb):
    """Pushforward pairs: depth 1 gives the one-step pairs bit for bit;
    at depth 2 the second input is one coarse step from the corrected
    first, and its target is the restricted fine state 8 fine steps on."""
    cr, m, _, _ = trained
    nfine, nc = (64, 64, 64), (32, 32, 32)
    X1, Y1 = cr.make_pairs(nfine, [21], 800, 100, 2)
    Xr, Yr = cr.make_rollout_pairs(m, nfine, [21], 800, 100, 2, 1)
    assert torch.equal(X1, Xr) and torch.equal(Y1, Yr)

    X2, Y2 = cr.make_rollout_pairs(m, nfine, [21], 800, 100, 1, 2)
    assert torch.equal(X2[0], X1[0]) and torch.equal(Y2[0], Y1[0])
    fine = cr._fine(nfine, 21, cr.FINE_PARAMS)
    fine.step(800)
    coarse = gb.BinaryFluid(nc, gb.FP32, **cr.coarse_params(cr.FINE_PARAMS))
    gb.coarse_restrict(fine, coarse)
    coarse.step(1)
    m.correct(coarse)
    coarse.step(1)
    fine.step(8)
    x = torch.empty_like(X2[1])
    y = torch.empty_like(Y2[1])
    gb.fields_pack(coarse, x.data_ptr())
    gb.fields_restrict(fine, y.data_ptr(), nc)
    gb.sync()
    assert torch.equal(x, X2[1]) and torch.equal(y, Y2[1])


def test_forward_n_matches_forward(trained):
    """Forward passes issued back to back give what single calls give."""
    cr, m, _, _ = trained
    N = m.nsites
    rng = np.random.default_rng(3)
    xs = [dev(0.1 * rng.standard_normal((5, N))) for _ in range(3)]
    outs = [torch.empty((4, N), dtype=torch.float32, device="cuda")
            for _ in range(3)]
    m.forward_n([x.data_ptr() for x in xs], [o.data_ptr() for o in outs])
    for x, o in zip(xs, outs):
        ref = torch.empty_like(o)
        m.forward(x.data_ptr(), ref.data_ptr())
        assert torch.equal(ref, o)


def test_forward_after_direct_convolution(gb, orc):
    """A direct convolution call packs its own 32-channel data into the
    first layer's input rows; the next forward pass must rewrite all 32
    channels (the feature kernel otherwise writes 16): the result equals
    that of a model that never made the call."""
    n = (2, 4, 128)
    N = n[0] * n[1] * n[2]
    rng = np.random.default_rng(5)
    m1, m2 = gb.Corrector(n, seed=3), gb.Corrector(n, seed=3)
    a = dev(rng.standard_normal((N, 32)))
    w = dev(0.2 * rng.standard_normal((27, 32, 32)))
    b = dev(rng.standard_normal(32))
    junk = torch.empty((N, 32), dtype=torch.float32, device="cuda")
    m1.conv3(a.data_ptr(), w.data_ptr(), b.data_ptr(), 0, junk.data_ptr())
    x = dev(0.1 * rng.standard_normal((5, N)))
    t = dev(0.1 * rng.standard_normal((4, N)))
    o1 = torch.empty((4, N), dtype=torch.float32, device="cuda")
    o2 = torch.empty_like(o1)
    m1.forward(x.data_ptr(), o1.data_ptr())
    m2.forward(x.data_ptr(), o2.data_ptr())
    assert torch.equal(o1, o2)
    # the weight gradient of the first layer reads all 32 input channels
    l1 = m1.loss_grad(x.data_ptr(), t.data_ptr())
    l2 = m2.loss_grad(x.data_ptr(), t.data_ptr())
    assert l1 == l2
    assert np.array_equal(m1.grads(), m2.grads())


@pytest.mark.parametrize("n", [(4, 4, 128), (3, 17, 128)])
def test_three_tap_forward_matches_one_tap(gb, n):
    """The network's forward pass in the three-tap line form (the last
    layer with 16 weight rows a tap) against the one-tap line form: the
    same products summed in another order.  The activations between the
    layers are rounded to BF16, where a last-bit difference of a sum can
    move a value by one BF16 step (2^-8 relative), so the outputs agree to
    the network oracle's tolerance, not to FP32 rounding."""
    N = n[0] * n[1] * n[2]
    rng = np.random.default_rng(21)
    m = gb.Corrector(n, seed=11)
    p = m.params()
    p[3 * 27680:3 * 27680 + 27648] *= 10.0
    m.set_params(p)
    x = dev(0.3 * rng.standard_normal((5, N)))
    outs = {}
    for mode in (1, 3, 4, 5):
        m.line_reuse(mode)
        o = torch.empty((4, N), dtype=torch.float32, device="cuda")
        m.forward(x.data_ptr(), o.data_ptr())
        outs[mode] = o
    d = (outs[3] - outs[1]).abs().max().item()
    assert d <= 1e-2 * outs[1].abs().max().item(), d
    # 4 differs from 3 in the last layer only, whose inputs are the same
    # BF16 activations: its sums in another order, FP32 rounding apart
    d = (outs[4] - outs[3]).abs().max().item()
    assert d <= 1e-5 * outs[3].abs().max().item(), d
    # 5: the hidden layers on swizzled lines, the same sums as 4
    assert torch.equal(outs[5], outs[4])


def test_bounded_wait_times_out_and_context_survives(gb):
    """Failure detection without a fault: a device wait that nothing
    satisfies gives up after its clock budget (about a second), raises the
    error word and returns; the host reads LUDWIG_GB_ETIMEOUT, and the
    context still runs a step afterwards."""
    import ctypes
    secs = ctypes.c_double()
    rc = gb.lib().ludwig_gb_selftest_bounded_wait(ctypes.byref(secs))
    assert rc == 5                      # LUDWIG_GB_ETIMEOUT
    assert b"bounded" in gb.lib().ludwig_gb_last_error()
    assert 0.2 < secs.value < 10.0, secs.value
    s = gb.BinaryFluid((16, 16, 32), precision=gb.FP32)
    s.phi.init_spinodal(5, 0.0, 0.02)
    s.step(4)
    assert np.isfinite(s.phi.stats()[0])

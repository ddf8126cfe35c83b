"""Ensembles: every box of one launch equals the same box run alone.

FP64 ensembles are compared bit for bit with single-box FP64 runs (which
are themselves bit-exact against the oracle); FP32 ensembles with single-box
FP32 runs (same per-site arithmetic, so also exact) and with FP64 within
the reduced-precision tolerance."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small_ensemble(gb, nbox=5):
    rng = np.random.default_rng(3)
    params = []
    for k in range(nbox):
        n = [int(rng.choice([8, 12, 16, 20])) for _ in range(3)]
        kappa = float(rng.uniform(0.02, 0.08))
        amag = float(rng.uniform(0.03, 0.1))
        mob = min(0.45, 1.0 / (12.0 * (12.0 * kappa + 2.0 * amag)))
        params.append(gb.box_param(n, eta=float(rng.uniform(0.02, 0.2)),
                                   a=-amag, b=amag, kappa=kappa, mobility=mob,
                                   seed=100 + k))
    return params


def single(gb, p, prec, nsteps):
    s = gb.BinaryFluid(tuple(p.ntotal), precision=prec, a=p.a, b=p.b,
                       kappa=p.kappa, mobility=p.mobility, eta=p.eta)
    s.phi.init_spinodal(p.seed, p.phi0, p.noise)
    s.step(nsteps)
    return s.state()


@pytest.mark.parametrize("prec", [0, 1])
def test_ensemble_boxes_equal_single_runs(gb, prec):
    params = small_ensemble(gb)
    ens = gb.Ensemble(params, precision=prec)
    ens.step(9)
    for b, p in enumerate(params):
        got = ens.box(b, f=True)
        ref = single(gb, p, prec, 9)
        for k in ("phi", "u", "rho", "f"):
            assert np.array_equal(got[k], ref[k]), (b, k)


def test_ensemble_fp64_matches_oracle(gb, orc):
    params = small_ensemble(gb, 3)
    ens = gb.Ensemble(params, precision=0)
    ens.step(6)
    for b, p in enumerate(params):
        L = tuple(p.ntotal)
        st = orc.BinaryState(L, orc.lb_init_rest(L),
                             orc.spinodal_init(L, p.seed, 0.0, 0.02))
        orc.binary_steps(st, orc.symm_param(p.a, p.b, p.kappa), p.mobility,
                         orc.collide_param_m10(p.eta), 6)
        assert np.array_equal(ens.box(b)["phi"], st.phi)


def test_autotune_keeps_state(gb):
    params = small_ensemble(gb, 4)
    a = gb.Ensemble(params, precision=1)
    b = gb.Ensemble(params, precision=1)
    a.step(4)
    b.step(4)
    best, ms = a.autotune(4)
    assert ms > 0 and best[1] in (4, 8, 16)
    a.step(5)
    b.step(5)
    for k in range(len(params)):
        assert np.array_equal(a.box(k)["phi"], b.box(k)["phi"])


def test_diverging_box_is_quarantined(gb):
    """A box made non-finite is taken out; the others are unaffected."""
    params = small_ensemble(gb, 4)
    a = gb.Ensemble(params, precision=1)
    b = gb.Ensemble(params, precision=1)
    a.step(3)
    b.step(3)
    phi = a.box(2)["phi"]
    phi[0, 1, 1, 1] = np.nan
    a.set_phi(2, phi)
    a.step(2)
    assert a.check() == 3
    assert not a.active(2)
    a.step(4)
    b.step(6)
    for k in (0, 1, 3):
        assert np.array_equal(a.box(k)["phi"], b.box(k)["phi"])
    n = sum(int(np.prod(params[k].ntotal)) for k in (0, 1, 3))
    assert a.sites() == n


def test_config3_fp32_per_box_error_vs_fp64(gb):
    """The 64-box uneven ensemble (edges from {32, 48, 64, 96} per axis,
    viscosity, kappa and A = -B drawn per box) in FP32-shifted against the
    same ensemble in FP64, box by box: max |dphi| and the relative mass
    drift of every FP32 box, which must stay within the reduced-precision
    bounds (mass drift at most 1e-10, the bound set for 10^4 steps)."""
    from ludwig_gb300.precision import ensemble_error
    res = ensemble_error(gb.ensemble_uneven_boxes(), 200)
    assert res["nbox"] == 64
    for r in res["boxes"]:
        assert r["max_abs_dphi"] < 1e-4, r
        assert r["mass_drift_rel"] < 1e-10, r
        assert r["mass_drift_rel_fp64"] < 1e-12, r

"""Reduced-precision forms of the binary-fluid step against FP64.

The symmetric binary fluid (A = -B = -0.0625, kappa = 0.04, M = 0.3) is run from the
same KISS99 spinodal initial condition in FP64 (the bit-exact form), in
FP32 with distributions stored as deviations from w_p rho0, and with
FP16 storage.  At fixed intervals it reports, for each reduced form:
max |phi - phi_FP64|, the relative drift of the total mass since step 0,
and the domain length L(t) from the structure factor next to FP64's.

    python -m ludwig_gb300.precision --size 256 --steps 10000 --every 1000
    python -m ludwig_gb300.precision --lc --size 128 --steps 5000 --every 500
    python -m ludwig_gb300.precision --ensemble --steps 1000

For ensembles (many boxes of uneven sizes and parameters in one launch),
every box of the FP32 ensemble is compared with the same box of an FP64
ensemble: max |phi - phi_FP64| and the relative mass drift since step 0.
"""

import argparse
import json
import time

import numpy as np

from . import FP16, FP32, FP64, BinaryFluid, LudwigGBError, load_library

PARAMS = dict(a=-0.0625, b=0.0625, kappa=0.04, mobility=0.3, eta=0.1)
SEED = 8361235


def _mass(s):
    """Total mass, or None once the state is no longer finite."""
    try:
        m = s.lb.moments()[0]
    except LudwigGBError:
        return None
    return m if np.isfinite(m) else None


def run(size, steps, every, params=PARAMS, seed=SEED, log=print):
    n = (size,) * 3 if np.isscalar(size) else tuple(size)
    systems = {}
    for name, prec in (("fp64", FP64), ("fp32", FP32), ("fp16", FP16)):
        s = BinaryFluid(n, prec, **params)
        s.phi.init_spinodal(seed, 0.0, 0.02)
        systems[name] = s
    mass0 = {k: s.lb.moments()[0] for k, s in systems.items()}
    recs = []
    t = 0
    while t < steps:
        k = min(every, steps - t)
        t0 = time.time()
        for s in systems.values():
            s.step(k)
        t += k
        m64 = _mass(systems["fp64"])
        if m64 is None:
            # The FP64 run (bit-exact with the reference) has diverged: the
            # parameters are unstable at this size; nothing to compare with.
            rec = {"step": t, "diverged": "fp64 (bit-exact path): mass "
                   "not finite"}
            recs.append(rec)
            if log:
                log(json.dumps(rec))
            break
        phi64 = systems["fp64"].phi.get()
        L64 = systems["fp64"].phi.length_from_sk()[0]
        rec = {"step": t, "L_fp64": L64,
               "mass_drift_fp64": (m64 - mass0["fp64"]) / mass0["fp64"]}
        for name in ("fp32", "fp16"):
            s = systems[name]
            m = _mass(s)
            if m is None:
                rec[name] = {"diverged": True}
                continue
            L = s.phi.length_from_sk()[0]
            rec[name] = {
                "max_abs_dphi": float(np.abs(s.phi.get() - phi64).max()),
                "mass_drift_rel": (m - mass0[name]) / mass0[name],
                "L": L, "L_rel_err": (L - L64) / L64}
        rec["wall_s"] = time.time() - t0
        recs.append(rec)
        if log:
            log(json.dumps(rec))
    return recs


LC_PARAMS = dict(a0=0.01, gamma=3.0, kappa0=0.01, kappa1=0.01, pitch=32.0,
                 xi=0.7, redshift=1.0, amplitude=-0.2)


def run_lc(size, steps, every, log=print):
    """Cholesteric LC (blue phase I, O8M start) in FP64 and FP32: max |dQ|
    and the total free energy of each run (evaluated in FP64 from its Q)
    at fixed intervals."""
    from . import LiquidCrystal
    n = (size,) * 3 if np.isscalar(size) else tuple(size)
    s64 = LiquidCrystal(n, eta=0.5, gamma_rot=0.5, precision=FP64,
                        **LC_PARAMS)
    s32 = LiquidCrystal(n, eta=0.5, gamma_rot=0.5, precision=FP32,
                        **LC_PARAMS)
    holder = LiquidCrystal(n, eta=0.5, gamma_rot=0.5, precision=FP64,
                           **LC_PARAMS)
    s64.init_o8m()
    s32.q.set(s64.q.get())
    recs = []
    t = 0
    while t < steps:
        k = min(every, steps - t)
        t0 = time.time()
        s64.step(k)
        s32.step(k)
        t += k
        q64 = s64.q.get()
        q32 = s32.q.get()
        f64 = s64.fe.fed_total()
        holder.q.set(q32)
        f32 = holder.fe.fed_total()
        rec = {"step": t, "max_abs_dq": float(np.abs(q32 - q64).max()),
               "max_abs_q": float(np.abs(q64).max()),
               "fed_fp64": f64, "fed_fp32": f32,
               "fed_rel_err": (f32 - f64) / abs(f64),
               "wall_s": time.time() - t0}
        recs.append(rec)
        if log:
            log(json.dumps(rec))
    return recs


def _box_mass(ens, b):
    """Total mass of one box: the sum of its distributions, in FP64 (the
    reference f of a reduced-precision box is w_p rho0 plus the stored
    deviation, converted exactly)."""
    f = ens.box(b, f=True)["f"]
    return float(np.sum(f, dtype=np.float64))


def ensemble_error(params, steps, log=None):
    """Per-box error of the FP32-shifted ensemble against the FP64 one after
    `steps` steps.  Returns one record a box (edges, max |dphi|, max |phi|,
    relative mass drift of the FP32 box since step 0 and of the FP64 box)
    and the maxima over the boxes."""
    from . import Ensemble
    e32 = Ensemble(params, precision=FP32)
    e64 = Ensemble(params, precision=FP64)
    m0 = [float(np.prod(p.ntotal)) * p.rho0 for p in params]
    e32.step(steps)
    e64.step(steps)
    boxes = []
    for b, p in enumerate(params):
        g32 = e32.box(b)
        g64 = e64.box(b)
        m32 = _box_mass(e32, b)
        m64 = _box_mass(e64, b)
        rec = {"box": b, "ntotal": list(p.ntotal),
               "max_abs_dphi": float(np.abs(g32["phi"] - g64["phi"]).max()),
               "max_abs_phi": float(np.abs(g64["phi"]).max()),
               "mass_drift_rel": abs(m32 - m0[b]) / m0[b],
               "mass_drift_rel_fp64": abs(m64 - m0[b]) / m0[b]}
        boxes.append(rec)
        if log:
            log(json.dumps(rec))
    e32.close()
    e64.close()
    return {"steps": steps, "nbox": len(params),
            "max_dphi_max": max(r["max_abs_dphi"] for r in boxes),
            "drift_max": max(r["mass_drift_rel"] for r in boxes),
            "drift_max_fp64": max(r["mass_drift_rel_fp64"] for r in boxes),
            "boxes": boxes}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--size", type=int, default=256)
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--every", type=int, default=1000)
    ap.add_argument("--out", default=None)
    ap.add_argument("--eta", type=float, default=PARAMS["eta"],
                    help="shear viscosity (binary fluid)")
    ap.add_argument("--mobility", type=float, default=PARAMS["mobility"],
                    help="mobility (binary fluid); the explicit 7-point "
                    "Cahn-Hilliard step needs M < 2/(12(2|A| + 12 kappa)) "
                    "once the domains saturate")
    ap.add_argument("--lc", action="store_true",
                    help="the cholesteric LC (FP64 vs FP32) instead")
    ap.add_argument("--ensemble", action="store_true",
                    help="the 64-box uneven ensemble (FP32 vs FP64 per box)")
    args = ap.parse_args(argv)
    load_library()
    if args.ensemble:
        from . import ensemble_uneven_boxes
        res = ensemble_error(ensemble_uneven_boxes(), args.steps,
                             log=print)
        res["model"] = "ensemble of 64 uneven binary-fluid boxes"
    elif args.lc:
        recs = run_lc(args.size, args.steps, args.every)
        res = {"model": "cholesteric LC", "size": args.size,
               "steps": args.steps, "params": LC_PARAMS, "records": recs}
    else:
        params = dict(PARAMS, eta=args.eta, mobility=args.mobility)
        recs = run(args.size, args.steps, args.every, params=params)
        res = {"size": args.size, "steps": args.steps, "params": params,
               "seed": SEED, "records": recs}
    if args.out:
        with open(args.out, "w") as f:
            json.dump(res, f, indent=1)
    return res


if __name__ == "__main__":
    main()

"""Learned corrector for a binary fluid run on a 2x-coarsened lattice.

The plain method on the fine lattice (FP32-shifted fused step) generates
the data: snapshots of fine runs are restricted to the coarse lattice
(diffusive scaling: dx x 2, dt x 4, so one coarse step stands for four
fine steps, velocities x 2, strain rates x 4), the coarse method takes one
step from each restricted state, and the network learns the difference
between that step and the restricted fine state four fine steps later.
At run time the network corrects phi and u after every coarse step.

Coarse parameters from the fine ones (same equations in coarse units):
A and B x 4, kappa unchanged (interface width / 2), mobility / 4,
viscosity unchanged.

Everything numeric runs on the GPU through libludwig_gb.so (the fused
step, the restriction kernels, the tensor-core network); torch tensors
only hold the snapshot pairs in device memory.

Command line (the full-size workload):

    python -m ludwig_gb300.corrector --fine 256 --seeds 16 --out DIR
"""

import argparse
import json
import math
import os
import time

import numpy as np

from . import (FP32, FP64, PE, BinaryFluid, Coords, Corrector, Field,
               coarse_restrict, fields_pack, fields_restrict, load_library,
               sync)

FINE_PARAMS = dict(a=-0.0625, b=0.0625, kappa=0.04, mobility=0.3, eta=0.1)


def coarse_params(p):
    """Parameters of the coarse lattice (diffusive scaling by 2)."""
    return dict(a=4.0 * p["a"], b=4.0 * p["b"], kappa=p["kappa"],
                mobility=p["mobility"] / 4.0, eta=p["eta"])


def _torch():
    import torch
    return torch


def _fine(nfine, seed, params, precision=FP32):
    s = BinaryFluid(nfine, precision, **params)
    s.phi.init_spinodal(seed, 0.0, 0.02)
    return s


def make_pairs(nfine, seeds, t_first, t_gap, npairs, params=FINE_PARAMS,
               log=None):
    """Snapshot pairs on the device.

    Returns (X, Y): X[i] = coarse fields [phi, u, rho] after one coarse step
    from the restricted fine state, Y[i] = restricted fine fields four fine
    steps later; both float32 tensors of shape [P, 5, Nc] on cuda:0.
    """
    torch = _torch()
    nc = tuple(n // 2 for n in nfine)
    Nc = nc[0] * nc[1] * nc[2]
    P = len(seeds) * npairs
    X = torch.empty((P, 5, Nc), dtype=torch.float32, device="cuda")
    Y = torch.empty((P, 5, Nc), dtype=torch.float32, device="cuda")
    coarse = BinaryFluid(nc, FP32, **coarse_params(params))
    i = 0
    for seed in seeds:
        t0 = time.time()
        fine = _fine(nfine, seed, params)
        fine.step(t_first)
        for k in range(npairs):
            coarse_restrict(fine, coarse)
            coarse.step(1)
            fields_pack(coarse, X[i].data_ptr())
            fine.step(4)
            fields_restrict(fine, Y[i].data_ptr(), nc)
            i += 1
            if k + 1 < npairs:
                fine.step(t_gap - 4)
        sync()
        del fine
        if log:
            log("pairs: seed %d done (%.1f s)" % (seed, time.time() - t0))
    return X, Y


def make_rollout_pairs(model, nfine, seeds, t_first, t_gap, nstarts, depth,
                       params=FINE_PARAMS, log=None):
    """Pairs along the corrected coarse run itself ("pushforward"): from
    each restricted fine state the coarse lattice takes `depth` steps,
    corrected by the current network after each but the last; step j's
    fields are paired with the restricted fine state 4 j fine steps after
    the start.  The network then learns to correct the states its own
    rollout reaches, error included, toward the fine trajectory (pairs of
    depth 1 are those of make_pairs).  Returns (X, Y) as make_pairs."""
    torch = _torch()
    nc = tuple(n // 2 for n in nfine)
    Nc = nc[0] * nc[1] * nc[2]
    P = len(seeds) * nstarts * depth
    X = torch.empty((P, 5, Nc), dtype=torch.float32, device="cuda")
    Y = torch.empty((P, 5, Nc), dtype=torch.float32, device="cuda")
    coarse = BinaryFluid(nc, FP32, **coarse_params(params))
    i = 0
    for seed in seeds:
        t0 = time.time()
        fine = _fine(nfine, seed, params)
        fine.step(t_first)
        for k in range(nstarts):
            coarse_restrict(fine, coarse)
            for j in range(depth):
                fine.step(4)
                fields_restrict(fine, Y[i].data_ptr(), nc)
                coarse.step(1)
                fields_pack(coarse, X[i].data_ptr())
                if j + 1 < depth:
                    sync()
                    model.correct(coarse)
                i += 1
            if k + 1 < nstarts:
                fine.step(t_gap - 4 * depth)
        sync()
        del fine
        if log:
            log("rollout pairs: seed %d done (%.1f s)"
                % (seed, time.time() - t0))
    return X, Y


def scales_from(X, Y):
    """Feature normalisation and target scales from the data."""
    x = X.double()
    d = (Y[:, :4] - X[:, :4]).double()
    off = [0.0, 0.0, 0.0, 0.0, 1.0]
    sphi = float(x[:, 0].std())
    su = float(x[:, 1:4].std())
    srho = float((x[:, 4] - 1.0).std())
    in_scale = [1.0 / max(sphi, 1e-12)] + [1.0 / max(su, 1e-12)] * 3 \
        + [1.0 / max(srho, 1e-12)]
    dphi = float(d[:, 0].std())
    du = float(d[:, 1:4].std())
    out_scale = [max(dphi, 1e-12)] + [max(du, 1e-12)] * 3
    return off, in_scale, out_scale


def targets(X, Y, out_scale):
    torch = _torch()
    s = torch.tensor(out_scale, dtype=torch.float32,
                     device=X.device).view(1, 4, 1)
    t = ((Y[:, :4] - X[:, :4]) / s).contiguous()
    torch.cuda.synchronize()          # the library reads it on its own stream
    return t


def train(model, X, T, epochs, lr=1e-3, seed=0, log=None):
    """Adam over the pairs, shuffled each epoch, cosine learning rate."""
    rng = np.random.default_rng(seed)
    P = X.shape[0]
    total = epochs * P
    k = 0
    hist = []
    for ep in range(epochs):
        order = rng.permutation(P)
        acc = 0.0
        for i in order:
            r = lr * 0.5 * (1.0 + math.cos(math.pi * k / total))
            acc += model.train_step(X[i].data_ptr(), T[i].data_ptr(),
                                    max(r, lr * 1e-2))
            k += 1
        hist.append(acc / P)
        if log:
            log("epoch %d: mean loss %.5f" % (ep, acc / P))
    return hist


def one_step_errors(model, X, T):
    """Mean normalised squared error without and with the network."""
    torch = _torch()
    out = torch.empty_like(T[0])
    base, corr = 0.0, 0.0
    for i in range(X.shape[0]):
        model.forward(X[i].data_ptr(), out.data_ptr())
        base += float((T[i] * T[i]).mean())
        d = out - T[i]
        corr += float((d * d).mean())
    n = X.shape[0]
    return base / n, corr / n


def restrict_phi(phi):
    """Average 2x2x2 blocks (numpy, any precision)."""
    p = np.asarray(phi)
    if p.ndim == 4:
        p = p[0]
    nx, ny, nz = p.shape
    return p.reshape(nx // 2, 2, ny // 2, 2, nz // 2, 2).mean(axis=(1, 3, 5))


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def rollout(model, nfine, seed, t0, ncoarse_steps, every, params=FINE_PARAMS,
            fine_precision=FP64, log=None):
    """Coarse runs with and without the network against the fine run.

    The fine run (fine_precision) starts from the seed; at fine step t0
    both coarse runs start from its restriction (an FP32 copy of it when
    the fine run is FP64 is not needed: the FP32 twin provides the state).
    Returns a list of records: coarse step, rel. L2 error of phi (plain,
    corrected), domain length L (fine restricted, plain, corrected).
    """
    nc = tuple(n // 2 for n in nfine)
    cp = coarse_params(params)
    fine = _fine(nfine, seed, params, fine_precision)
    twin = _fine(nfine, seed, params, FP32)
    fine.step(t0)
    twin.step(t0)
    plain = BinaryFluid(nc, FP32, **cp)
    corr = BinaryFluid(nc, FP32, **cp)
    coarse_restrict(twin, plain)
    coarse_restrict(twin, corr)
    del twin
    ref_cs = Coords(PE(0), nc)                 # holder for L of R(phi_f)
    ref_phi = Field(ref_cs, 1, 2, FP64, "phi")
    out = []
    for k in range(1, ncoarse_steps + 1):
        fine.step(4)
        plain.step(1)
        corr.step(1)
        model.correct(corr)
        if k % every == 0 or k == ncoarse_steps:
            pf = restrict_phi(fine.phi.get())
            pp = plain.phi.get()[0]
            pc = corr.phi.get()[0]
            ref_phi.set(pf.reshape((1,) + pf.shape).astype(np.float64))
            rec = {"coarse_step": k, "fine_step": t0 + 4 * k,
                   "err_plain": rel_l2(pp, pf), "err_corrected": rel_l2(pc, pf),
                   "L_fine": ref_phi.length_from_sk()[0],
                   "L_plain": plain.phi.length_from_sk()[0],
                   "L_corrected": corr.phi.length_from_sk()[0]}
            out.append(rec)
            if log:
                log("rollout %s" % json.dumps(rec))
    return out


# Executed forward work of the default convolution forms, in units of a
# 32 -> 32 layer: the first layer reads 16 input channels (0.5); where
# nz = 128 the last layer runs folded, 3 MMAs of N = 48 per y-line and 18
# y-lines per 16 outputs (0.1875 of a layer), else as a full layer.
def default_exec_layers(nz):
    return 2.5 + 0.1875 if nz == 128 else 3.5


def time_network(model, x, t, reps=20, exec_layers=3.5):
    """Time per forward pass and per training step (forward, backward,
    Adam) on one pair, issued back to back (`forward_n`, `train_steps`:
    one error check per batch), the same with one call and one host check
    per pass ("call"), and the tensor-core work they carry."""
    torch = _torch()
    out = torch.empty_like(t)
    model.forward(x.data_ptr(), out.data_ptr())
    sync()
    t0 = time.perf_counter()
    for _ in range(reps):
        model.forward(x.data_ptr(), out.data_ptr())
    sync()
    fwd_call = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    model.forward_n([x.data_ptr()] * reps, [out.data_ptr()] * reps)
    sync()
    fwd = (time.perf_counter() - t0) / reps
    lr = 1e-12
    model.train_step(x.data_ptr(), t.data_ptr(), lr)
    t0 = time.perf_counter()
    for _ in range(reps):
        model.train_step(x.data_ptr(), t.data_ptr(), lr)
    sync()
    step_call = (time.perf_counter() - t0) / reps
    t0 = time.perf_counter()
    model.train_steps([x.data_ptr()] * reps, [t.data_ptr()] * reps, lr)
    sync()
    step = (time.perf_counter() - t0) / reps
    n = model.nsites
    # executed MMA work: 4 convolutions forward in units of a 32 -> 32
    # layer (exec_layers; default_exec_layers gives it for the default
    # forms), 3 backward-data and 4 weight gradients (28 of 27 taps)
    flop_conv = 2.0 * n * 27 * 32 * 32
    flop_fwd = exec_layers * flop_conv
    flop_step = flop_fwd + 3 * flop_conv + 4 * flop_conv * 28.0 / 27.0
    return {"sites": n, "forward_ms": 1e3 * fwd, "train_step_ms": 1e3 * step,
            "forward_call_ms": 1e3 * fwd_call,
            "train_step_call_ms": 1e3 * step_call,
            "forward_tflops": flop_fwd / fwd / 1e12,
            "train_step_tflops": flop_step / step / 1e12,
            "note": "forward_ms, train_step_ms: wall time per pass of a "
                    "batch issued back to back; *_call_ms: one call and "
                    "one host check per pass"}


def bench(n, reps=20):
    """Forward and training-step times of the network on synthetic inputs
    (n^3 coarse sites), per-tap and line-reuse convolutions."""
    torch = _torch()
    g = torch.Generator(device="cuda").manual_seed(1)
    N = n ** 3
    model = Corrector((n, n, n), seed=1)
    x = 0.1 * torch.randn((5, N), device="cuda", generator=g)
    x[4] += 1.0
    t = 0.1 * torch.randn((4, N), device="cuda", generator=g)
    torch.cuda.synchronize()
    # executed layers (in 32 x 32 layers): the three-tap last layer
    # computes 16 weight rows a tap (0.5), the folded one (the default
    # where nz = 128) 0.1875
    three = (n == 128)
    folded = default_exec_layers(128)
    res = {"default": time_network(model, x, t, reps,
                                   default_exec_layers(n))}
    for mode, name in ((0, "per_tap"), (1, "line_planes"),
                       (2, "line_swizzled"), (3, "line_three_taps"),
                       (4, "line_folded_last"),
                       (5, "line_three_taps_swizzled")):
        model.line_reuse(mode)
        ex = 3.5
        if three and mode == 3:
            ex = 3.0
        if three and mode in (4, 5):
            ex = folded
        res[name] = time_network(model, x, t, reps, ex)
    return res


def choose_method(records, tol=0.02):
    """The corrected coarse run is used only where its phi error stays
    within tol of the fine run; otherwise the plain fine lattice is used."""
    worst = max(r["err_corrected"] for r in records)
    return ("coarse+corrector" if worst <= tol else "fine"), worst


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--fine", type=int, default=256)
    ap.add_argument("--seeds", type=int, default=16)
    ap.add_argument("--holdout", type=int, default=2)
    ap.add_argument("--t-first", type=int, default=1000)
    ap.add_argument("--t-gap", type=int, default=100)
    ap.add_argument("--pairs", type=int, default=13)
    ap.add_argument("--epochs", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--rollout", type=int, default=250)
    ap.add_argument("--every", type=int, default=25)
    ap.add_argument("--pushforward", type=int, default=0,
                    help="after the first training, pairs along the "
                    "corrected coarse run of this depth (coarse steps), "
                    "then training on them (0: none)")
    ap.add_argument("--pf-starts", type=int, default=4,
                    help="rollout starts per seed for the pushforward pairs")
    ap.add_argument("--pf-rounds", type=int, default=1)
    ap.add_argument("--pf-epochs", type=int, default=4)
    ap.add_argument("--out", default="corrector_out")
    ap.add_argument("--bench", type=int, default=0,
                    help="only time the network on a BENCH^3 coarse lattice")
    ap.add_argument("--reps", type=int, default=20)
    args = ap.parse_args(argv)

    load_library()
    if args.bench:
        res = bench(args.bench, args.reps)
        print(json.dumps(res))
        return res
    os.makedirs(args.out, exist_ok=True)
    logf = open(os.path.join(args.out, "log.txt"), "w")

    def log(msg):
        print(msg, flush=True)
        logf.write(msg + "\n")
        logf.flush()

    if 4 * args.pushforward > args.t_gap:
        ap.error("--pushforward %d needs --t-gap >= %d"
                 % (args.pushforward, 4 * args.pushforward))
    nfine = (args.fine,) * 3
    nc = tuple(n // 2 for n in nfine)
    seeds = [1000 + s for s in range(args.seeds)]
    hold = [2000 + s for s in range(args.holdout)]
    t = time.time()
    X, Y = make_pairs(nfine, seeds, args.t_first, args.t_gap, args.pairs,
                      log=log)
    t_data = time.time() - t
    off, isc, osc = scales_from(X, Y)
    T = targets(X, Y, osc)
    model = Corrector(nc, seed=12345)
    model.set_scales(off, isc, osc)
    base0, corr0 = one_step_errors(model, X, T)
    t = time.time()
    hist = train(model, X, T, args.epochs, args.lr, log=log)
    sync()
    t_train = time.time() - t
    base1, corr1 = one_step_errors(model, X, T)
    timing = time_network(model, X[0], T[0],
                          exec_layers=default_exec_layers(model.n[2]))
    log("timing %s" % json.dumps(timing))
    del X, Y, T
    pf_hist = []
    for rnd in range(args.pushforward and args.pf_rounds):
        # rollout stability: train on the states the corrected rollout
        # reaches (scales kept from the first data set)
        t = time.time()
        Xr, Yr = make_rollout_pairs(model, nfine, seeds, args.t_first,
                                    args.t_gap, args.pf_starts,
                                    args.pushforward, log=log)
        Tr = targets(Xr, Yr, osc)
        pf_hist.append(train(model, Xr, Tr, args.pf_epochs, args.lr * 0.3,
                             seed=1 + rnd, log=log))
        sync()
        log("pushforward round %d: %.1f s" % (rnd, time.time() - t))
        del Xr, Yr, Tr
    hb = hc = None
    if hold:
        Xh, Yh = make_pairs(nfine, hold, args.t_first, args.t_gap,
                            args.pairs)
        Th = targets(Xh, Yh, osc)
        hb, hc = one_step_errors(model, Xh, Th)
        del Xh, Yh, Th
    recs, method, worst = [], None, None
    if hold and args.rollout > 0:
        recs = rollout(model, nfine, hold[0], args.t_first, args.rollout,
                       args.every, log=log)
        method, worst = choose_method(recs)
    np.save(os.path.join(args.out, "params.npy"), model.params())
    res = {"fine": list(nfine), "coarse": list(nc), "pairs": len(seeds) *
           args.pairs, "seeds": len(seeds), "holdout_seeds": hold,
           "epochs": args.epochs, "data_s": t_data, "train_s": t_train,
           "train_steps": args.epochs * len(seeds) * args.pairs,
           "loss_history": hist, "pushforward_depth": args.pushforward,
           "pushforward_rounds": args.pushforward and args.pf_rounds,
           "pushforward_loss_history": pf_hist,
           "one_step_train": {"plain": base1, "corrected": corr1,
                              "initial_network": corr0},
           "one_step_holdout": {"plain": hb, "corrected": hc},
           "rollout": recs, "method_chosen": method, "timing": timing,
           "worst_rollout_error": worst,
           "scales": {"in_off": off, "in_scale": isc, "out_scale": osc}}
    with open(os.path.join(args.out, "result.json"), "w") as f:
        json.dump(res, f, indent=1)
    log(json.dumps({k: res[k] for k in ("one_step_holdout", "method_chosen",
                                        "worst_rollout_error", "train_s")}))
    return res


if __name__ == "__main__":
    main()

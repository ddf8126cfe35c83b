"""Benchmark: D3Q19 symmetric binary fluid at 256^3 on one GB300.

Workload (one "step" = one time step of the main loop of the reference,
src/ludwig.c:528-860, for the symmetric free energy: 7-point gradients,
stress-divergence force, upwind + chemical-potential Cahn-Hilliard fluxes,
forward-Euler phi update, M10 collision with the force, streaming):
  256^3 periodic, rho0 = 1, eta = 0.1, A = -0.0625, B = 0.0625,
  kappa = 0.04, M = 0.3, phi0 uniform in [-0.01, 0.01] from the reference's
  KISS99 per-site seeding (seed 8361235), f at rest equilibrium.

Headline ``value``: MLUPS of the FP32-shifted fused step (float arithmetic,
f stored as f - w_p rho0), inputs resident in HBM; the state (3.1 GB) is
larger than L2, so no flush is needed between steps.  Beside it: the FP64
fused step (bit-identical to the reference's arithmetic) and the FP16-storage
form, the end-to-end rate through the C ABI with the state in pinned host
memory, and the CPU oracle on the host cores.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Under torchrun (N > 1) every rank runs an independent replica of the box on
its own GPU ("replicas only": the single-box path has no exchange step);
``value`` is the total over ranks divided by the slowest rank's time.
"""

import argparse
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SIZE = (256, 256, 256)
LEGS = ("fp32", "e2e", "fp16", "fp64", "dropin", "lb2", "lc", "ens", "cnn",
        "cpu")
PARAMS = dict(a=-0.0625, b=0.0625, kappa=0.04, mobility=0.3, eta=0.1)
SEED = 8361235
METRIC = "D3Q19 binary-fluid MLUPS at 256^3, FP32-shifted (FP64 beside it)"

# Algorithmic bytes per site update (compulsory traffic of the fused step):
#   FP64: f 2*19*8 + phi 2*8 + u 2*3*8 = 368;  FP32: 184;  FP16: f 2*19*2 +
#   phi 2*4 + u 2*12 = 108.  rho (written for output) is not counted.
ALGO_BYTES = {"fp64": 368, "fp32": 184, "fp16": 108,
              # cholesteric LC: f 2*19 + Q 2*5 + u 2*3 values per site
              "lc64": 432, "lc32": 216}

# Algorithmic bytes per site of one step through the per-function C API in
# the main-loop order (each kernel reads its input arrays once and writes
# its outputs once; intermediates stored as the reference stores them):
# binary fluid FP64: hydro_f_zero 24, gradient 40 (phi -> grad, delsq),
# stress 112 (phi, grad, delsq -> P), force divergence 120 (P, force r/w),
# upwind fluxes 64 (phi, u -> 4 fluxes), chemical-potential fluxes 80
# (phi, delsq, 4 fluxes r/w), phi update 48 (4 fluxes, phi r/w),
# hydro_u_zero 24, collision pulling the pending propagation 360 (f, force
# -> f, rho, u) = 872.  Cholesteric FP64: 24 + gradients 200 (Q -> 15
# gradients, 5 Laplacians) + stress 272 + force 120 + upwind fluxes 224
# (Q, u -> 20 fluxes) + molecular field 240 (Q, gradients -> H) +
# Beris-Edwards 304 (u, 20 fluxes, H, Q r/w) + 24 + 360 = 1768.
DROPIN_BYTES = {"dropin_binary64": 872, "dropin_lc64": 1768,
                # symmetric_lb (two distributions), one step of three
                # kernels: phi from g (g 152 -> phi 8), gradients (phi 8 ->
                # grad 24, delsq 8), collision pulling f and g (f, g 304,
                # phi, grad, delsq 40 -> f, g 304, u 24) = 872
                "lb2_64": 872}

# DRAM bytes (read + write) per site of the fused kernels, from one ncu
# capture each (binary fluid at 160^3, cholesteric at 128^3; the fused
# float LC step is two kernels, 32.5 + 35.0 + 112.2 + 72.0); a streaming
# kernel's traffic grows in proportion to the sites, so traffic =
# bytes/site x sites.
NCU_BYTES_PER_SITE = {"fp32": 179.8, "fp64": 370.5, "fp16": 103.4,
                      "lc32": 251.7}

# Corrector FLOPs per coarse site and forward pass (3x3x3 convolutions):
# executed as 4 layers of 32 x 32 channels, 2*27*32*32 each; useful are
# the real layer shapes 5 -> 32 -> 32 -> 32 -> 4: 2*27*(5*32 + 2*32*32 +
# 32*4) = 126,144.
# executed per site: first layer K = 16; the last layer in the folded
# form at 128^3, 3 MMAs (dx) of N = 48 and K = 32 per y-line, 18 y-lines
# per run of 16 output lines
CNN_EXEC_FLOP = 2 * 27 * (16 * 32 + 32 * 32 + 32 * 32) + \
    2 * 3 * 48 * 32 * 18 // 16
CNN_USEFUL_FLOP = 2 * 27 * (5 * 32 + 2 * 32 * 32 + 32 * 4)

# What bounds each kernel (ncu): the FP64 form is FP64-pipe bound.
LIMITER = {"fp32": "hbm (traffic = compulsory bytes; issue 65% busy)",
           "dropin_binary64": "one kernel per reference function, FP64 "
                              "(--fmad=false); intermediates through HBM",
           "dropin_lc64": "one kernel per reference function, FP64; "
                          "intermediates through HBM",
           "fp64": "fp64 pipe (83.5% active at 160^3, ncu)",
           "fp16": "two sites per thread in packed FP32x2, next plane's "
                   "populations prefetched; issue and dependency waits at "
                   "12 warps per SM (108 B/site)",
           "lc64": "fp64 pipe",
           "lb2_64": "fp64 pipe (two collisions a site, --fmad=false)",
           "lc32": "two kernels: fields + Beris-Edwards (issue and load "
                   "latency), force + collision (HBM: stress neighbours "
                   "through L1, 91% of the measured copy bandwidth); the "
                   "stress (9 values a site) crosses HBM between them"}


def env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fp:
            d = json.load(fp)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,"
              "clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device),
                 "--query-gpu=" + self.FIELDS,
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            out, _ = self.proc.communicate(timeout=5)
        except Exception:
            self.proc.kill()
            out, _ = self.proc.communicate()
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in out.strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax = max(smax, float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax,
                "samples": len(sm), "reasons": sorted(reasons)}


def dist_setup():
    world = env_int("WORLD_SIZE", 1)
    rank = env_int("RANK", 0)
    local = env_int("LOCAL_RANK", 0)
    pg = None
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
        pg = dist
    return world, rank, local, pg


def barrier(pg):
    if pg is not None:
        pg.barrier()


def max_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(pg, v):
    if pg is None:
        return v
    import torch
    t = torch.tensor([float(v)], dtype=torch.float64)
    pg.all_reduce(t, op=pg.ReduceOp.SUM)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU legs: the oracle (a C restatement of the reference), host cores
# ---------------------------------------------------------------------------

def cpu_run(size, steps, threads):
    """MLUPS of the oracle on the host cores (test infrastructure)."""
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle
    oracle.build()
    fe = oracle.symm_param(PARAMS["a"], PARAMS["b"], PARAMS["kappa"])
    cp = oracle.collide_param_m10(PARAMS["eta"])
    st = oracle.BinaryState(size, oracle.lb_init_rest(size),
                            oracle.spinodal_init(size, SEED, 0.0, 0.02))
    oracle.binary_steps(st, fe, PARAMS["mobility"], cp, 1)   # warm-up
    t0 = time.perf_counter()
    oracle.binary_steps(st, fe, PARAMS["mobility"], cp, steps)
    dt = time.perf_counter() - t0
    n = size[0] * size[1] * size[2]
    return n * steps / dt / 1e6, dt


def reference_arm(args):
    world, rank, local, pg = dist_setup()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    # Each step: one oracle step on a 256 x 256 x 16 periodic slab, 1/16 of
    # the 256^3 workload with the same per-site work and a working set
    # (~0.5 GB) far beyond the caches.
    sample = (SIZE[0], SIZE[1], 16)
    os.environ["OMP_NUM_THREADS"] = str(threads)
    import oracle
    oracle.build()
    fe = oracle.symm_param(PARAMS["a"], PARAMS["b"], PARAMS["kappa"])
    cp = oracle.collide_param_m10(PARAMS["eta"])
    st = oracle.BinaryState(sample, oracle.lb_init_rest(sample),
                            oracle.spinodal_init(sample, SEED, 0.0, 0.02))
    oracle.binary_steps(st, fe, PARAMS["mobility"], cp, args.warmup)
    t0 = time.perf_counter()
    oracle.binary_steps(st, fe, PARAMS["mobility"], cp, args.steps)
    dt = time.perf_counter() - t0
    n = sample[0] * sample[1] * sample[2]
    mlups = n * args.steps / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": mlups,
        "unit": "MLUPS", "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * dt / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (spinodal phi0, seed %d)" % SEED,
        "config": {"workload": "symmetric binary fluid 256^3, M10, 7pt, "
                   "FD Cahn-Hilliard", "size": list(SIZE),
                   "precision": "fp64"},
        "cpu_baseline": {"value": mlups, "unit": "MLUPS", "cores": threads,
                         "kind": "port",
                         "sample": "%d steps of a 256x256x16 periodic slab "
                                   "(1/16 of 256^3), oracle C restatement, "
                                   "OpenMP" % args.steps},
        "e2e": {"value": mlups, "unit": "MLUPS", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------

def make_system(lg, prec):
    s = lg.BinaryFluid(SIZE, precision=prec, a=PARAMS["a"], b=PARAMS["b"],
                       kappa=PARAMS["kappa"], mobility=PARAMS["mobility"],
                       eta=PARAMS["eta"])
    s.phi.init_spinodal(SEED, 0.0, 0.02)
    return s


def roofline(kind, ms_per_step, nsites, peak, peak_kind):
    algo = (ALGO_BYTES.get(kind) or DROPIN_BYTES[kind]) * nsites
    achieved = algo / (ms_per_step * 1e-3) / 1e9
    ncu = NCU_BYTES_PER_SITE.get(kind)
    if kind not in LIMITER:
        raise KeyError(kind)
    return {"bound": "hbm", "achieved": achieved, "peak": peak,
            "unit": "GB/s", "frac": achieved / peak,
            "traffic": None if ncu is None else ncu * nsites,
            "algorithmic_bytes": algo, "limiter": LIMITER[kind],
            "peak_source": "%s (MEASURED_PEAKS.json hbm_gbs)" % peak_kind
            if peak_kind == "measured" else "fallback 6.8 TB/s"}


def gpu_arm(args):
    world, rank, local, pg = dist_setup()
    import ludwig_gb300 as lg
    lg.load_library()
    lg.PE(local)                      # select the device for this rank
    lg.tune_sites(args.sites)
    nsites = SIZE[0] * SIZE[1] * SIZE[2]
    peak, peak_kind = measured_peaks()

    # --- headline: FP32-shifted -------------------------------------------
    s32 = make_system(lg, lg.FP32)
    s32.step(args.warmup)
    lg.sync()
    m0 = s32.lb.moments()[0]
    clocks = Clocks(local)
    clocks.start()
    barrier(pg)
    lg.sync()
    ms32 = lg.time_binary(s32, args.steps)
    lg.sync()
    barrier(pg)
    clk = clocks.stop()
    ms32 = max_over_ranks(pg, ms32)
    m1 = s32.lb.moments()[0]
    drift32 = abs(m1 - m0) / m0 / args.steps
    phi_stats32 = s32.phi.stats()

    legs = set(args.legs.split(","))

    # --- end to end through the C ABI with host buffers --------------------
    e2e_steps = max(3, min(args.steps, 20))
    ms_e2e, h2d, d2h = float("nan"), 0, 0
    ms_e2e_serial = float("nan")
    if "e2e" in legs:
        # every step: upload the state from pinned host memory, one fused
        # step, download the result; the copies of consecutive steps overlap
        pin_in, pin_out = lg.PinnedState(s32), lg.PinnedState(s32)
        lg.time_binary_e2e_overlap(s32, pin_in, pin_out, 2)    # warm-up
        barrier(pg)
        ms_e2e = lg.time_binary_e2e_overlap(s32, pin_in, pin_out, e2e_steps)
        barrier(pg)
        ms_e2e = max_over_ranks(pg, ms_e2e)
        h2d, d2h = pin_in.bytes_in, pin_out.bytes_out
        # the same, each step's copies and step in sequence on one stream
        lg.time_binary_e2e(s32, pin_in, 1)
        ms_e2e_serial = lg.time_binary_e2e(s32, pin_in, e2e_steps)
        pin_in.close()
        pin_out.close()
    s32 = None

    # --- FP16 storage -------------------------------------------------------
    ms16 = float("nan")
    if "fp16" in legs:
        s16 = make_system(lg, lg.FP16)
        s16.step(args.warmup)
        lg.sync()
        ms16 = lg.time_binary(s16, args.steps)
        s16 = None

    # --- FP64 (reference-exact arithmetic) ---------------------------------
    k64 = max(2, min(args.steps, 40))
    ms64 = float("nan")
    if "fp64" in legs:
        s64 = make_system(lg, lg.FP64)
        s64.step(min(args.warmup, 3))
        lg.sync()
        barrier(pg)
        ms64 = lg.time_binary(s64, k64)
        barrier(pg)
        ms64 = max_over_ranks(pg, ms64)
        s64 = None

    # --- the drop-in path: one C-API call per reference function ---------
    dropin = None
    if "dropin" in legs:
        dropin = {}
        sb = make_system(lg, lg.FP64)
        sb.step_reference_order(2)
        lg.sync()
        kd = 10
        t0 = time.perf_counter()
        sb.step_reference_order(kd)
        lg.sync()
        dt = time.perf_counter() - t0
        dropin["binary_fp64"] = {
            "value": nsites * kd / dt / 1e6, "unit": "MLUPS", "steps": kd,
            "ms_per_step": 1e3 * dt / kd,
            "roofline": roofline("dropin_binary64", 1e3 * dt / kd, nsites, peak,
                                 peak_kind),
            "workload": "256^3 binary fluid FP64, per step: hydro_f_zero, "
                        "field_halo, field_grad_compute, "
                        "phi_force_calculation, hydro_u_halo, "
                        "phi_cahn_hilliard, hydro_u_zero, lb_collide, "
                        "lb_halo, lb_propagation (each call synchronous), "
                        "host wall time"}
        sb = None
        n_lc = (128, 128, 128)
        slc = lg.LiquidCrystal(n_lc, eta=0.5, gamma_rot=0.5,
                               precision=lg.FP64)
        slc.init_o8m()
        slc.step_reference_order(2)
        lg.sync()
        t0 = time.perf_counter()
        slc.step_reference_order(kd)
        lg.sync()
        dt = time.perf_counter() - t0
        sites_lc = 128 ** 3
        dropin["lc_fp64"] = {
            "value": sites_lc * kd / dt / 1e6, "unit": "MLUPS", "steps": kd,
            "ms_per_step": 1e3 * dt / kd,
            "roofline": roofline("dropin_lc64", 1e3 * dt / kd, sites_lc, peak,
                                 peak_kind),
            "workload": "128^3 cholesteric BP I FP64, per step: "
                        "hydro_f_zero, field_halo, field_grad_compute, "
                        "phi_force_calculation, hydro_u_halo, "
                        "beris_edw_update, hydro_u_zero, lb_collide, "
                        "lb_halo, lb_propagation, host wall time"}
        slc = None

    # --- symmetric_lb (order parameter as a second distribution), FP64 ----
    lb2 = None
    if "lb2" in legs:
        n2 = (128, 128, 128)
        s2 = lg.BinaryFluidLB(n2, a=PARAMS["a"], b=PARAMS["b"],
                              kappa=PARAMS["kappa"], mobility=0.45,
                              eta=PARAMS["eta"])
        s2.init_spinodal(SEED, 0.0, 0.02)
        s2.step(3)
        lg.sync()
        k2 = 10
        t0 = time.perf_counter()
        s2.step(k2)
        lg.sync()
        dt = time.perf_counter() - t0
        sites2 = 128 ** 3
        lb2 = {"value": sites2 * k2 / dt / 1e6, "unit": "MLUPS", "steps": k2,
               "ms_per_step": 1e3 * dt / k2,
               "roofline": roofline("lb2_64", 1e3 * dt / k2, sites2, peak,
                                    peak_kind),
               "workload": "128^3 binary fluid with symmetric_lb (ndist=2, "
                           "M=0.45), FP64 bit-exact, 3 kernels a step, host "
                           "wall time"}
        s2 = None

    # --- cholesteric LC (blue phase I), 128^3, FP32 and FP64 ------------
    lc = None
    if "lc" in legs:
        lc = {}
        n_lc = (128, 128, 128)
        sites_lc = 128 ** 3
        for name, prec, k in (("fp32", lg.FP32, max(args.steps // 4, 10)),
                              ("fp64", lg.FP64, 10)):
            slc = lg.LiquidCrystal(n_lc, eta=0.5, gamma_rot=0.5,
                                   precision=prec)
            slc.init_o8m()
            slc.step(3)
            ms = slc.time(k)
            kind = "lc32" if name == "fp32" else "lc64"
            lc[name] = {"value": sites_lc * k / (ms * 1e-3) / 1e6,
                        "unit": "MLUPS", "steps": k, "ms_per_step": ms / k,
                        "roofline": roofline(kind, ms / k, sites_lc, peak,
                                             peak_kind)}
            slc = None
        lc["workload"] = ("cholesteric LC 128^3, O8M blue phase I, pitch 32, "
                          "A0=0.01 gamma=3 kappa0=kappa1=0.01 xi=0.7 "
                          "Gamma=0.5 eta=0.5, two kernels per step")

    # --- ensemble of 64 uneven boxes, FP32, one persistent launch -------
    ens = None
    if "ens" in legs:
        # the 64 boxes are shared out over the ranks (no exchange between
        # boxes); one rank runs them all
        from ludwig_gb300 import shard
        boxes = lg.ensemble_uneven_boxes()
        mine = shard.shard_boxes(boxes, world)[rank]
        e = lg.Ensemble([boxes[i] for i in mine], precision=lg.FP32)
        best, _ = e.autotune(10)
        ke = max(args.steps // 4, 20)
        barrier(pg)
        ms = e.time(ke)
        barrier(pg)
        ms = max_over_ranks(pg, ms)
        sites_all = sum_over_ranks(pg, e.sites())
        ens = {"value": sites_all * ke / (ms * 1e-3) / 1e6, "unit": "MLUPS",
               "steps": ke, "ms_per_step": ms / ke, "sites": sites_all,
               "tiling": {"xchunk": best[0], "tile_y": best[1],
                          "min_blocks": best[2]},
               "ranks": world,
               "workload": "64 periodic boxes, edges from {32,48,64,96}, "
                           "per-box parameters, FP32-shifted, one launch "
                           "per step under a CUDA graph; boxes shared out "
                           "over the ranks by size"}
        e.close()
        # config 3's per-box error: every FP32 box against the same box
        # run in FP64, after the same number of steps
        from ludwig_gb300.precision import ensemble_error
        ksteps = 200
        err = ensemble_error([boxes[i] for i in mine], ksteps)
        ens["per_box_error"] = {
            "steps": ksteps, "boxes": err["nbox"],
            "max_dphi_max": err["max_dphi_max"],
            "drift_max": err["drift_max"],
            "drift_max_fp64": err["drift_max_fp64"],
            "how": "FP32-shifted ensemble vs FP64 ensemble of the same "
                   "boxes: max over boxes of max|dphi| and of the relative "
                   "mass drift since step 0"}

    # --- learned corrector on the 128^3 coarse lattice --------------------
    cnn = None
    if "cnn" in legs:
        try:
            from ludwig_gb300.corrector import bench as cnn_bench
            r = cnn_bench(128, reps=max(3, min(args.steps // 20, 20)))
            d = r["default"]
            fwd = d["forward_ms"]
            ncs = 128 ** 3
            cnn = {"forward_ms": fwd,
                   "train_step_ms": d["train_step_ms"],
                   "forward_call_ms": d["forward_call_ms"],
                   "train_step_call_ms": d["train_step_call_ms"],
                   "forward_tflops": d["forward_tflops"],
                   "forward_tflops_useful":
                       CNN_USEFUL_FLOP * ncs / (fwd * 1e-3) / 1e12,
                   "useful_over_executed": CNN_USEFUL_FLOP / CNN_EXEC_FLOP,
                   "train_step_tflops": d["train_step_tflops"],
                   "forward_ms_by_form": {k: v["forward_ms"]
                                          for k, v in r.items()},
                   "unit_note": "forward_tflops: executed BF16 MMA work "
                                "(layers of 32x32 channels, the first "
                                "with 16 input channels, the last as "
                                "3 MMAs of N = 48 per y-line) / wall "
                                "time per "
                                "pass, passes issued back to back; "
                                "forward_tflops_useful: the real layer "
                                "shapes 5-32-32-32-4; *_call_ms: one call "
                                "and one host check per pass",
                   "workload": "4-layer 3x3x3 conv net, 32 channels, 128^3 "
                               "coarse lattice, tcgen05 BF16 / FP32"}
        except ImportError as exc:                   # torch missing
            cnn = {"unavailable": str(exc)}

    total_sites = sum_over_ranks(pg, nsites)
    per32 = ms32 / args.steps
    value = total_sites * args.steps / (ms32 * 1e-3) / 1e6
    fp64_mlups = total_sites * k64 / (ms64 * 1e-3) / 1e6
    fp16_mlups = nsites * args.steps / (ms16 * 1e-3) / 1e6 * world
    e2e = total_sites * e2e_steps / (ms_e2e * 1e-3) / 1e6
    e2e_serial = nsites * e2e_steps / (ms_e2e_serial * 1e-3) / 1e6

    if cnn is not None and "forward_ms" in cnn and ms32 == ms32:
        # one coarse step (128^3, a quarter of the fine step's sites x 1/2
        # per axis) plus one forward pass stands for 4 fine steps at 256^3
        per32_fine = ms32 / args.steps
        coarse_ms = per32_fine / 8.0
        cnn["cost_ratio_vs_4_fine_steps"] = (
            (coarse_ms + cnn["forward_ms"]) / (4.0 * per32_fine))
        cnn["cost_note"] = ("(coarse FP32 step, estimated as 1/8 of the "
                            "fine step, + forward) / (4 fine FP32 steps "
                            "at 256^3); < 1 means the corrected coarse run "
                            "is cheaper")

    if rank != 0:
        return 0

    cpu = None
    try:
        if "cpu" not in legs:
            raise RuntimeError("leg not run")
        threads = os.cpu_count() or 1
        cpu_mlups, cpu_dt = cpu_run(SIZE, 2, threads)
        cpu = {"value": cpu_mlups, "unit": "MLUPS", "cores": threads,
               "kind": "port",
               "sample": "2 steps at 256^3 after 1 warm-up step (%.1f s), "
                         "oracle C restatement of the reference, OpenMP"
                         % cpu_dt}
    except Exception as exc:                          # pragma: no cover
        cpu = {"value": None, "unit": "MLUPS", "cores": 0, "kind": "port",
               "sample": "failed: %s" % exc}

    line = {
        "metric": METRIC, "value": value, "unit": "MLUPS", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": per32,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic: spinodal phi0 in [-0.01,0.01] (KISS99 seed %d), "
                "f at rest" % SEED,
        "config": {"workload": "symmetric binary fluid 256^3 periodic, D3Q19 "
                   "M10, 7-point gradients, stress divergence, FD "
                   "Cahn-Hilliard (A=-0.0625 B=0.0625 kappa=0.04 M=0.3 "
                   "eta=0.1)", "size": list(SIZE),
                   "precision": "fp32-shifted",
                   "l2": "state larger than L2 (3.1 GB), no flush",
                   "parallelism": "replicas" if world > 1 else "1 GPU"},
        "roofline": roofline("fp32", per32, nsites, peak, peak_kind),
        "cpu_baseline": cpu,
        "e2e": {"value": e2e, "unit": "MLUPS", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "how": "per step: f, phi, u H2D from pinned host memory, one "
                       "fused step, f, phi, u, rho D2H (C ABI); two device "
                       "buffer sets so that the upload of step k+1 overlaps "
                       "the download of step k",
                "serial": {"value": e2e_serial, "unit": "MLUPS",
                           "how": "the same with copies and step in "
                                  "sequence on one stream"}},
        "gpu_launches": args.steps,
        "clocks": clk,
        "fp64": {"value": fp64_mlups, "unit": "MLUPS", "steps": k64,
                 "ms_per_step": ms64 / k64,
                 "vs_cpu_baseline": (fp64_mlups / cpu["value"]
                                     if cpu and cpu.get("value") else None),
                 "vs_cpu_note": "FP64 on both sides: the bit-exact GPU step "
                                "over cpu_baseline (the oracle, FP64)",
                 "roofline": roofline("fp64", ms64 / k64, nsites, peak,
                                      peak_kind)},
        "fp16": {"value": fp16_mlups, "unit": "MLUPS",
                 "ms_per_step": ms16 / args.steps,
                 "roofline": roofline("fp16", ms16 / args.steps, nsites, peak,
                                      peak_kind)},
        "dropin": dropin,
        "lb2": lb2,
        "lc": lc,
        "ensemble": ens,
        "corrector": cnn,
        "fp32_over_fp64": value / fp64_mlups,
        "mass_drift_rel_per_step_fp32": drift32,
        "phi_stats_fp32": [float(v) for v in phi_stats32],
    }
    print(json.dumps(_finite(line)), flush=True)
    return 0


def _finite(obj):
    """Replace NaN/Inf (legs not run) by null so the line is strict JSON."""
    if isinstance(obj, dict):
        return {k: _finite(v) for k, v in obj.items()}
    if isinstance(obj, list):
        return [_finite(v) for v in obj]
    if isinstance(obj, float) and not np.isfinite(obj):
        return None
    return obj


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--size", type=int, default=256,
                    help="lattice edge (default 256; smaller for profiling)")
    ap.add_argument("--sites", type=int, default=0, choices=[0, 1, 2],
                    help="sites per thread of the float fused step (0: the "
                    "faster form of each precision)")
    ap.add_argument("--legs", default=",".join(LEGS),
                    help="comma list of %s" % ",".join(LEGS))
    args = ap.parse_args()
    global SIZE
    SIZE = (args.size,) * 3
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)
    return gpu_arm(args)


if __name__ == "__main__":
    sys.exit(main())

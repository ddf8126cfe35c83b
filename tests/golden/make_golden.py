"""Generate the golden fixtures of tests/golden/ from the reference itself.

The reference (Ludwig v0.23) is built from its own sources into
oracle/_ref by oracle/ref.mk, and oracle/ref_shim.c drives its hot-path
functions (lb_collide, lb_propagation, field_grad_compute,
phi_force_calculation, phi_cahn_hilliard and the main-loop step of
src/ludwig.c) on seeded inputs.  Inputs and outputs are saved as .npz.

Needs the reference sources (only where they are present):
    python tests/golden/make_golden.py [/path/to/reference]
(default: $LUDWIG_REFERENCE_ROOT, else REF of oracle/ref.mk) [--only=lb2|grad27|logs|advection|io|config1|length]
"""

import hashlib
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402

SYMM = dict(A=-0.0625, B=0.0625, K=0.04, M=0.3, eta=0.1)


def kv(L, **extra):
    d = dict(size="%d,%d,%d" % L)
    d.update({k: repr(v) if isinstance(v, float) else str(v)
              for k, v in extra.items()})
    return d


def sha256_of(a):
    """SHA-256 of an array's values as little-endian doubles in C order: a
    compact bit-for-bit pin of a field too large to commit whole."""
    return hashlib.sha256(np.ascontiguousarray(a, "<f8").tobytes()).hexdigest()


def run_case(name, L, steps, seed, status=None, keep=("phi", "u", "rho",
                                                       "force", "f"),
             hashed=(), **extra):
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "out")
        args = kv(L, mode="run", steps=steps, seed=seed, noise=0.02,
                  phi0=0.0, out=out, dump0=1, **SYMM, **extra)
        if status is not None:
            sp = os.path.join(tmp, "status.bin")
            status.astype(np.uint8).tofile(sp)
            args["status"] = sp
        oracle.run_reference(args)
        res = {"L": np.array(L), "steps": steps, "seed": seed}
        for k, v in extra.items():
            res[k] = v
        if status is not None:
            res["status"] = status.astype(np.uint8)
        res["phi0"] = oracle.read_array(out + "0", "phi", (1,) + L)
        ncomp = dict(phi=1, u=3, rho=1, force=3, f=19)
        for k in keep:
            res[k] = oracle.read_array(out, k, (ncomp[k],) + L)
        for k in hashed:
            res["sha256_" + k] = np.array(
                sha256_of(oracle.read_array(out, k, (ncomp[k],) + L)))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
    print("wrote", name)


def op_case(name, mode, L, inputs, outputs, **extra):
    with tempfile.TemporaryDirectory() as tmp:
        pin, pout = os.path.join(tmp, "in"), os.path.join(tmp, "out")
        oracle.write_arrays(pin, **inputs)
        oracle.run_reference(kv(L, mode=mode, **{"in": pin}, out=pout,
                                **SYMM, **extra))
        res = {"L": np.array(L)}
        res.update({"in_" + k: v for k, v in inputs.items()})
        for k, nc in outputs.items():
            res[k] = oracle.read_array(pout, k, (nc,) + L)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
    print("wrote", name)


LC = dict(a0=0.01, gamma=3.0, kappa0=0.01, kappa1=0.01, pitch=32.0, xi=0.7,
          Gamma=0.5, redshift=1.0, amplitude=-0.2, eta=0.5)


def lc_run_case(name, L, steps):
    """Blue phase I (o8m) initial condition, then the LC main loop."""
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "out")
        oracle.run_reference(kv(L, mode="lc", steps=steps, out=out, **LC))
        res = {"L": np.array(L), "steps": steps}
        res["q0"] = oracle.read_array(out, "q0", (5,) + L)
        for k, nc in (("q", 5), ("u", 3), ("rho", 1), ("force", 3),
                      ("f", 19)):
            res[k] = oracle.read_array(out, k, (nc,) + L)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
    print("wrote", name)


def lc_op_case(name, mode, L, inputs, outputs):
    with tempfile.TemporaryDirectory() as tmp:
        pin, pout = os.path.join(tmp, "in"), os.path.join(tmp, "out")
        oracle.write_arrays(pin, **inputs)
        oracle.run_reference(kv(L, mode=mode, **{"in": pin}, out=pout, **LC))
        res = {"L": np.array(L)}
        res.update({"in_" + k: v for k, v in inputs.items()})
        for k, nc in outputs.items():
            res[k] = oracle.read_array(pout, k, (nc,) + L)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
    print("wrote", name)


LB2 = dict(A=-0.0625, B=0.0625, K=0.04, M=0.45, eta=0.1)


def lb2_run_case(name, L, steps, seed):
    """symmetric_lb (two distributions): spinodal phi moved into g, then
    the main loop with ndist = 2; mobility 0.45 (stable on this route)."""
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "out")
        oracle.run_reference(kv(L, mode="lb2", ndist=2, steps=steps,
                                seed=seed, noise=0.02, phi0=0.0, out=out,
                                **LB2))
        res = {"L": np.array(L), "steps": steps, "seed": seed}
        for k, nc in (("phi", 1), ("u", 3), ("f", 19), ("g", 19)):
            res[k] = oracle.read_array(out, k, (nc,) + L)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
    print("wrote", name)


def lb2_cases():
    rng = np.random.default_rng(20261204)
    lb2_run_case("lb2_8x6x4_s10", (8, 6, 4), 10, 8361235)
    lb2_run_case("lb2_12x10x8_s60", (12, 10, 8), 60, 91)
    L = (6, 5, 4)
    f = oracle.lb_init_rest(L) * (1.0 + 1e-3 * rng.standard_normal((19,) + L))
    phi = rng.uniform(-1, 1, (1,) + L)
    g = 1e-2 * rng.standard_normal((19,) + L)
    g[0] = phi[0] - g[1:].sum(axis=0)
    with tempfile.TemporaryDirectory() as tmp:
        pin, pout = os.path.join(tmp, "in"), os.path.join(tmp, "out")
        oracle.write_arrays(pin, f=f, g=g, phi=phi)
        oracle.run_reference(kv(L, mode="collide2", ndist=2, **{"in": pin},
                                out=pout, **LB2))
        res = {"L": np.array(L), "in_f": f, "in_g": g, "in_phi": phi}
        for k, nc in (("f", 19), ("g", 19), ("u", 3)):
            res[k] = oracle.read_array(pout, k, (nc,) + L)
    np.savez_compressed(os.path.join(HERE, "collide2_6x5x4.npz"), **res)
    print("wrote collide2_6x5x4")


def grad27_cases():
    rng = np.random.default_rng(20261205)
    L = (6, 5, 4)
    for nf in (1, 5):
        a = rng.uniform(-1, 1, (nf,) + L)
        with tempfile.TemporaryDirectory() as tmp:
            pin, pout = os.path.join(tmp, "in"), os.path.join(tmp, "out")
            oracle.write_arrays(pin, phi=a)
            oracle.run_reference(kv(L, mode="grad27", nf=nf, **{"in": pin},
                                    out=pout))
            res = {"L": np.array(L), "in_phi": a}
            res["grad"] = oracle.read_array(pout, "grad", (3 * nf,) + L)
            res["delsq"] = oracle.read_array(pout, "delsq", (nf,) + L)
        name = "grad27_nf%d_6x5x4" % nf
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print("wrote", name)


REGRESSION_LOGS = ("serial-spin-fd1", "serial-spin-lb1", "serial-init-bp1",
                   "serial-symm-dr1", "serial-init-bp2", "serial-relx-bp1",
                   "serial-chol-fld", "serial-init-br1", "serial-init-br2",
                   "serial-symm-pat", "serial-init-lcr", "serial-init-lcb",
                   "d3q19-io/iodrop-mpi1-io1", "d3q19-io/iodrop-mpi1-io3")


def parse_log(path):
    """Statistics blocks of a reference regression log: a list (initial
    conditions, then each statistics step) of {tag: [numbers]}."""
    blocks, cur = [], None
    for line in open(path):
        t = line.strip()
        if t.startswith("Initial conditions") or \
                t.startswith("Starting time step loop") or \
                t.startswith("Completed cycle"):
            if cur:
                blocks.append(cur)
            cur = {}
            continue
        if cur is None or not t.startswith("["):
            continue
        tag, rest = t[1:].split("]", 1)
        vals = []
        for w in rest.split():
            try:
                vals.append(float(w))
            except ValueError:
                pass
        if vals:
            cur.setdefault(tag.strip(), vals)
    if cur:
        blocks.append(cur)
    return [b for b in blocks if b]


def regression_logs(ref_root):
    """Numbers of the reference's own regression logs for the cases this
    path covers (read as text), into tests/golden/regression_logs.json."""
    import json
    d = os.path.join(ref_root, "tests", "regression")
    out = {}
    for name in REGRESSION_LOGS:
        sub = name if "/" in name else "d3q19-short/" + name
        out[name.split("/")[-1]] = parse_log(os.path.join(d, sub + ".log"))
    with open(os.path.join(HERE, "regression_logs.json"), "w") as f:
        json.dump(out, f, indent=1)
    print("wrote regression_logs.json")


def advection_cases():
    """Runs with the 2nd- and 3rd-order advective fluxes and the 27-point
    gradient (src/advection.c, src/gradient_3d_27pt_fluid.c)."""
    run_case("run_adv2_8x6x4_s10", (8, 6, 4), 10, 8361235, order=2)
    run_case("run_adv3_12x10x8_s30", (12, 10, 8), 30, 77, order=3)
    run_case("run_adv2_g27_10x8x6_s12", (10, 8, 6), 12, 4242, order=2,
             grad=27)
    run_case("run_adv3_g27_8x8x8_s20", (8, 8, 8), 20, 99, order=3, grad=27)


IO_CASES = (("io_d1_phi_bin", (3, 2, 2), 1, 1, "binary", 10, 1),
            ("io_d2_phi_asc", (3, 2, 2), 2, 1, "ascii", 20, 1),
            ("io_d1_q_asc", (2, 3, 2), 1, 5, "ascii", 0, 0),
            ("io_d1_q_bin", (4, 2, 3), 1, 5, "binary", 123456789, 0))


def io_cases():
    """Snapshot files written by the reference's lb_io_write and
    field_io_write (src/lb_data.c:1716, src/field.c:1633), with the
    arrays that went in; each file's bytes are kept."""
    rng = np.random.default_rng(20251)
    for name, L, ndist, nf, fmt, step, hydro in IO_CASES:
        n = L[0] * L[1] * L[2]
        f = (rng.standard_normal((ndist * 19,) + L) * 0.05
             + 1.0 / 19.0)
        q = rng.standard_normal((nf,) + L) * 0.3
        q.flat[0] = 1.0e-300          # exponent with three digits
        rho = 1.0 + 0.01 * rng.standard_normal((1,) + L)
        u = 0.02 * rng.standard_normal((3,) + L)
        with tempfile.TemporaryDirectory() as tmp:
            pin = os.path.join(tmp, "in")
            oracle.write_arrays(pin, f=f, phi=q, rho=rho, u=u)
            d = os.path.join(tmp, "files")
            os.mkdir(d)
            oracle.run_reference(kv(L, mode="io_write", ndist=ndist, nf=nf,
                                    fmt=fmt, step=step, dir=d, hydro=hydro,
                                    **{"in": pin}))
            res = {"L": np.array(L), "ndist": ndist, "nf": nf, "fmt": fmt,
                   "step": step, "in_f": f, "in_phi": q, "hydro": hydro}
            if hydro:
                res.update(in_rho=rho, in_u=u)
            names = sorted(os.listdir(d))
            res["files"] = np.array(names)
            for k, fn in enumerate(names):
                with open(os.path.join(d, fn), "rb") as fh:
                    res["file%d" % k] = np.frombuffer(fh.read(), np.uint8)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **res)
        print("wrote", name, n, "sites", names)


def length_fields(L=(128, 128, 128)):
    """Order-parameter fields for the L(t) fixtures that need no
    transcendental function (so that any machine builds the same doubles):
    a sphere of radius 24 (phi = 1 inside, -1 outside, by integer squared
    distance) and lamellae of period 16 along x."""
    x, y, z = np.meshgrid(*(np.arange(n) for n in L), indexing="ij")
    c = [n // 2 for n in L]
    r2 = (x - c[0]) ** 2 + (y - c[1]) ** 2 + (z - c[2]) ** 2
    sphere = np.where(r2 < 24 * 24, 1.0, -1.0)
    lamellae = np.where((x // 8) % 2 == 0, 1.0, -1.0)
    return {"sphere_r24": sphere[None], "lamellae_p16": lamellae[None]}


def length_cases():
    """The reference's util/length_from_sk.c (unmodified, compiled against
    oracle/fftw_api by oracle/ref.mk; it reads 128^3 binary phi files) on
    four 128^3 fields: the spinodal start (seed 8361235), the reference's
    own binary-fluid run from it after 600 steps (config 1's parameters),
    a sphere and lamellae.  Saved: the printed L (as printed, "%g") and the
    SHA-256 of each field's doubles; the fields are rebuilt by the test."""
    L = (128, 128, 128)
    exe = os.path.join(ROOT, "oracle", "_ref", "length_from_sk")
    res = {"L": np.array(L)}
    with tempfile.TemporaryDirectory() as tmp:
        out = os.path.join(tmp, "out")
        oracle.run_reference(kv(L, mode="run", steps=600, seed=8361235,
                                noise=0.02, phi0=0.0, out=out, dump0=1,
                                **SYMM), threads=os.cpu_count())
        fields = {"spinodal_s0": oracle.read_array(out + "0", "phi", (1,) + L),
                  "spinodal_s600": oracle.read_array(out, "phi", (1,) + L)}
        fields.update(length_fields(L))
        names = []
        for name, phi in fields.items():
            path = os.path.join(tmp, name)
            np.ascontiguousarray(phi, "<f8").tofile(path)
            txt = subprocess.run([exe, path], capture_output=True, text=True,
                                 check=True).stdout.strip()
            # "L = <file> <value>"
            res["L_" + name] = np.array(float(txt.split()[-1]))
            res["printed_" + name] = np.array(txt.split()[-1])
            res["sha256_" + name] = np.array(sha256_of(phi))
            names.append(name)
            print(name, txt.split()[-1])
        res["names"] = np.array(names)
    np.savez_compressed(os.path.join(HERE, "length_from_sk_128cube.npz"), **res)
    print("wrote length_from_sk_128cube")


def main(ref_root, only=None):
    if not oracle.build_reference(ref_root):
        raise SystemExit("reference sources not found at " + ref_root)
    if only == "lb2":
        lb2_cases()
        return
    if only == "grad27":
        grad27_cases()
        return
    if only == "logs":
        regression_logs(ref_root)
        return
    if only == "advection":
        advection_cases()
        return
    if only == "io":
        io_cases()
        return
    if only == "length":
        length_cases()
        return
    if only == "config1":
        run_case("run_32cube_s1000", (32, 32, 32), 1000, 8361235,
                 keep=("phi",), hashed=("f", "u", "rho", "force"))
        return
    rng = np.random.default_rng(20261203)

    run_case("run_8x6x4_s10", (8, 6, 4), 10, 8361235)
    run_case("run_12x10x8_s50", (12, 10, 8), 50, 77,
             keep=("phi", "u", "rho", "f"))
    st = (rng.uniform(size=(10, 8, 6)) < 0.1).astype(np.uint8)
    run_case("run_map_10x8x6_s12", (10, 8, 6), 12, 4242, status=st,
             keep=("phi", "u", "f"))
    run_case("run_32cube_s1000", (32, 32, 32), 1000, 8361235, keep=("phi",),
             hashed=("f", "u", "rho", "force"))

    L = (6, 5, 4)
    f = oracle.lb_init_rest(L) * (1.0 + 1e-3 * rng.standard_normal((19,) + L))
    force = 1e-4 * rng.standard_normal((3,) + L)
    op_case("collide_6x5x4", "collide", L, dict(f=f, force=force),
            dict(f=19, rho=1, u=3))
    L = (5, 4, 3)
    op_case("propagate_5x4x3", "propagate", L,
            dict(f=rng.standard_normal((19,) + L)), dict(f=19))
    L = (6, 5, 4)
    phi = rng.uniform(-1, 1, (1,) + L)
    op_case("grad_6x5x4", "grad", L, dict(phi=phi), dict(grad=3, delsq=1))
    op_case("force_6x5x4", "force", L, dict(phi=phi), dict(force=3))
    u = 0.01 * rng.standard_normal((3,) + L)
    op_case("ch_6x5x4", "ch", L, dict(phi=phi, u=u), dict(phi=1))

    lc_run_case("lc_8x8x8_s3", (8, 8, 8), 3)
    lc_run_case("lc_16x12x8_s40", (16, 12, 8), 40)
    L = (6, 5, 4)
    qbp = oracle.lc_init_o8m(L, oracle.lc_param())
    q = qbp + 0.01 * rng.standard_normal(qbp.shape)
    lc_op_case("lc_fields_6x5x4", "lc_fields", L, dict(q=q),
               dict(h=5, stress=9, fed=1))
    u = 0.005 * rng.standard_normal((3,) + L)
    lc_op_case("lc_be_6x5x4", "lc_be", L, dict(q=q, u=u), dict(q=5))
    lb2_cases()
    grad27_cases()
    advection_cases()
    io_cases()
    length_cases()
    regression_logs(ref_root)


if __name__ == "__main__":
    args = [a for a in sys.argv[1:] if not a.startswith("--only=")]
    only = [a[7:] for a in sys.argv[1:] if a.startswith("--only=")]
    main(args[0] if args else oracle.reference_root(),
         only[0] if only else None)

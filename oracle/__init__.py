"""CPU oracle for the lattice-Boltzmann hot path (test infrastructure only).

This package is the checker: a plain-C restatement (``ludwig_oracle.c``) of
the reference's algorithm, loaded through ctypes.  Only ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU legs import it; the
product library never does.

Array layout everywhere: interior sites only, periodic, component-major,
z fastest, i.e. numpy shape ``(ncomp, Lx, Ly, Lz)``, C order, float64.
"""

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")
REF_SHIM = os.path.join(REF_DIR, "ref_shim")

NVEL = 19

_lib = None


def build(quiet=True):
    """Compile the oracle shared library (gcc, -ffp-contract=off)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)


def reference_root():
    """Where the reference's sources are: $LUDWIG_REFERENCE_ROOT, else the
    default REF of the build recipe oracle/ref.mk."""
    env = os.environ.get("LUDWIG_REFERENCE_ROOT")
    if env:
        return env
    with open(os.path.join(HERE, "ref.mk")) as fh:
        for line in fh:
            if line.startswith("REF") and "?=" in line:
                return line.split("?=", 1)[1].strip()
    return ""


def build_reference(ref_root=None, jobs=8):
    """Build the reference itself (serial+OpenMP) into oracle/_ref.

    Only possible where the reference sources are present; used to pin the
    oracle and to regenerate golden fixtures.
    """
    if ref_root is None:
        ref_root = reference_root()
    if not ref_root or not os.path.isdir(ref_root):
        return False
    out = subprocess.run(["make", "-f", os.path.join(HERE, "ref.mk"),
                          "REF=" + ref_root, "-j%d" % jobs],
                         capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("reference build failed:\n" + out.stderr[-4000:])
    return True


class SymmParam(ctypes.Structure):
    _fields_ = [("a", ctypes.c_double), ("b", ctypes.c_double),
                ("kappa", ctypes.c_double)]


class CollideParam(ctypes.Structure):
    _fields_ = [("rtau_shear", ctypes.c_double),
                ("rtau_bulk", ctypes.c_double),
                ("rtau_ghost", ctypes.c_double * NVEL),
                ("force_global", ctypes.c_double * 3)]


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        _lib = ctypes.CDLL(LIB_PATH)
        _declare(_lib)
    return _lib


_P = ctypes.POINTER(ctypes.c_double)
_U8 = ctypes.POINTER(ctypes.c_uint8)
_I3 = ctypes.c_int * 3


def _declare(L):
    L.orc_collide_param_m10.argtypes = [ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double,
                                        ctypes.POINTER(CollideParam)]
    L.orc_spinodal_init.argtypes = [_I3, ctypes.c_int, ctypes.c_double,
                                    ctypes.c_double, _P]
    L.orc_lb_init_rest.argtypes = [_I3, ctypes.c_double, _P]
    L.orc_grad_7pt.argtypes = [_I3, ctypes.c_int, _P, _P, _P]
    L.orc_symm_mu.argtypes = [_I3, ctypes.POINTER(SymmParam), _P, _P, _P]
    L.orc_symm_stress.argtypes = [_I3, ctypes.POINTER(SymmParam), _P, _P, _P,
                                  _P]
    L.orc_force_divergence.argtypes = [_I3, _P, _P]
    L.orc_advect_upwind.argtypes = [_I3, ctypes.c_int, _P, _P, _P, _P, _P, _P]
    L.orc_ch_flux_mu.argtypes = [_I3, ctypes.POINTER(SymmParam),
                                 ctypes.c_double, _P, _P, _P, _P, _P, _P]
    L.orc_flux_no_normal.argtypes = [_I3, ctypes.c_int, _U8, _P, _P, _P, _P]
    L.orc_ch_update.argtypes = [_I3, _P, _P, _P, _P, _P]
    L.orc_collide_mrt.argtypes = [_I3, ctypes.POINTER(CollideParam), _U8, _P,
                                  _P, _P, _P]
    L.orc_propagate.argtypes = [_I3, _P, _P]
    L.orc_binary_step.argtypes = [_I3, ctypes.POINTER(SymmParam),
                                  ctypes.c_double,
                                  ctypes.POINTER(CollideParam), _U8,
                                  _P, _P, _P, _P, _P, _P, _P, ctypes.c_int]
    L.orc_field_stats.argtypes = [_I3, _P, _P]
    L.orc_symm_fed_total.argtypes = [_I3, ctypes.POINTER(SymmParam), _P, _P]
    L.orc_symm_fed_total.restype = ctypes.c_double
    for name in ("orc_ma", "orc_mi", "orc_wv"):
        getattr(L, name).restype = _P
    L.orc_cv.restype = ctypes.POINTER(ctypes.c_int8)


def _p(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_P)


def _u8(a):
    if a is None:
        return None
    assert a.dtype == np.uint8 and a.flags.c_contiguous
    return a.ctypes.data_as(_U8)


def _dims(L):
    return _I3(*[int(v) for v in L])


def tables():
    """(cv[19,3], wv[19], ma[19,19], mi[19,19]) as used by the oracle."""
    L = lib()
    cv = np.ctypeslib.as_array(L.orc_cv(), shape=(NVEL * 3,)).reshape(NVEL, 3)
    wv = np.ctypeslib.as_array(L.orc_wv(), shape=(NVEL,))
    ma = np.ctypeslib.as_array(L.orc_ma(), shape=(NVEL * NVEL,))
    mi = np.ctypeslib.as_array(L.orc_mi(), shape=(NVEL * NVEL,))
    return (cv.copy(), wv.copy(), ma.reshape(NVEL, NVEL).copy(),
            mi.reshape(NVEL, NVEL).copy())


def collide_param_m10(eta, eta_bulk=None, rho0=1.0, force_global=(0, 0, 0)):
    p = CollideParam()
    lib().orc_collide_param_m10(float(eta), float(eta if eta_bulk is None
                                                  else eta_bulk),
                                float(rho0), ctypes.byref(p))
    for i in range(3):
        p.force_global[i] = float(force_global[i])
    return p


def symm_param(a, b, kappa):
    return SymmParam(float(a), float(b), float(kappa))


def spinodal_init(L, seed, phi0=0.0, amp=0.02):
    phi = np.zeros((1,) + tuple(L))
    lib().orc_spinodal_init(_dims(L), int(seed), float(phi0), float(amp),
                            _p(phi))
    return phi


def lb_init_rest(L, rho0=1.0):
    f = np.zeros((NVEL,) + tuple(L))
    lib().orc_lb_init_rest(_dims(L), float(rho0), _p(f))
    return f


def grad_7pt(L, field):
    field = np.ascontiguousarray(field, dtype=np.float64)
    nf = field.shape[0]
    grad = np.zeros((3 * nf,) + tuple(L))
    delsq = np.zeros((nf,) + tuple(L))
    lib().orc_grad_7pt(_dims(L), nf, _p(field), _p(grad), _p(delsq))
    return grad, delsq


def grad_27pt(L, field):
    """src/gradient_3d_27pt_fluid.c:219-362 (fluid sites only)."""
    field = np.ascontiguousarray(field, dtype=np.float64)
    nf = field.shape[0]
    grad = np.zeros((3 * nf,) + tuple(L))
    delsq = np.zeros((nf,) + tuple(L))
    Lb = lib()
    Lb.orc_grad_27pt.argtypes = [_I3, ctypes.c_int, _P, _P, _P]
    Lb.orc_grad_27pt(_dims(L), nf, _p(field), _p(grad), _p(delsq))
    return grad, delsq


def symm_stress(L, fe, phi, grad, delsq):
    pth = np.zeros((9,) + tuple(L))
    lib().orc_symm_stress(_dims(L), ctypes.byref(fe), _p(phi), _p(grad),
                          _p(delsq), _p(pth))
    return pth


def symm_mu(L, fe, phi, delsq):
    mu = np.zeros((1,) + tuple(L))
    lib().orc_symm_mu(_dims(L), ctypes.byref(fe), _p(phi), _p(delsq), _p(mu))
    return mu


def force_divergence(L, pth, force=None):
    if force is None:
        force = np.zeros((3,) + tuple(L))
    lib().orc_force_divergence(_dims(L), _p(pth), _p(force))
    return force


def phi_force(L, fe, phi):
    """phi_force_calculation (stress divergence) on a zeroed force."""
    grad, delsq = grad_7pt(L, phi)
    pth = symm_stress(L, fe, phi, grad, delsq)
    return force_divergence(L, pth)


def cahn_hilliard(L, fe, mobility, phi, u, status=None):
    """phi_cahn_hilliard: returns the updated phi (a copy)."""
    phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
    u = np.ascontiguousarray(u, dtype=np.float64)
    grad, delsq = grad_7pt(L, phi)
    fw, fe_, fy, fz = (np.zeros((1,) + tuple(L)) for _ in range(4))
    lib().orc_advect_upwind(_dims(L), 1, _p(phi), _p(u), _p(fw), _p(fe_),
                            _p(fy), _p(fz))
    lib().orc_ch_flux_mu(_dims(L), ctypes.byref(fe), float(mobility), _p(phi),
                         _p(delsq), _p(fw), _p(fe_), _p(fy), _p(fz))
    lib().orc_flux_no_normal(_dims(L), 1, _u8(status), _p(fw), _p(fe_),
                             _p(fy), _p(fz))
    lib().orc_ch_update(_dims(L), _p(fw), _p(fe_), _p(fy), _p(fz), _p(phi))
    return phi


def collide(L, cp, f, force, status=None):
    """lb_collide (M10): returns (f, rho, u); f is a copy."""
    f = np.ascontiguousarray(f, dtype=np.float64).copy()
    force = np.ascontiguousarray(force, dtype=np.float64)
    rho = np.zeros((1,) + tuple(L))
    u = np.zeros((3,) + tuple(L))
    lib().orc_collide_mrt(_dims(L), ctypes.byref(cp), _u8(status), _p(f),
                          _p(force), _p(rho), _p(u))
    return f, rho, u


def propagate(L, f):
    f = np.ascontiguousarray(f, dtype=np.float64)
    out = np.zeros_like(f)
    lib().orc_propagate(_dims(L), _p(f), _p(out))
    return out


class BinaryState:
    """Host state of the binary fluid: f, phi, u, rho, force."""

    def __init__(self, L, f, phi, u=None):
        self.L = tuple(int(v) for v in L)
        n = self.L
        self.f = np.ascontiguousarray(f, dtype=np.float64).copy()
        self.phi = np.ascontiguousarray(phi, dtype=np.float64).copy()
        self.u = (np.zeros((3,) + n) if u is None else
                  np.ascontiguousarray(u, dtype=np.float64).copy())
        self.rho = np.zeros((1,) + n)
        self.force = np.zeros((3,) + n)
        self._fs = np.zeros_like(self.f)
        self._work = np.zeros((13,) + n)


def binary_steps(state, fe, mobility, cp, nsteps, status=None):
    """Advance a BinaryState by nsteps of the reference main loop."""
    s = state
    lib().orc_binary_step(_dims(s.L), ctypes.byref(fe), float(mobility),
                          ctypes.byref(cp), _u8(status), _p(s.f), _p(s._fs),
                          _p(s.phi), _p(s.u), _p(s.rho), _p(s.force),
                          _p(s._work), int(nsteps))
    return s


class Lb2State:
    """Host state of the two-distribution binary fluid: f, g, phi, u."""

    def __init__(self, L, f, g, phi=None):
        self.L = tuple(int(v) for v in L)
        n = self.L
        self.f = np.ascontiguousarray(f, dtype=np.float64).copy()
        self.g = np.ascontiguousarray(g, dtype=np.float64).copy()
        self.phi = (np.zeros((1,) + n) if phi is None else
                    np.ascontiguousarray(phi, dtype=np.float64).copy())
        self.u = np.zeros((3,) + n)
        self._scratch = np.zeros_like(self.f)
        self._work = np.zeros((4,) + n)


def lb2_g_from_phi(phi):
    """src/phi_lb_coupler.c:107-135: phi into g_0, the other g_p zero."""
    phi = np.asarray(phi, dtype=np.float64)
    g = np.zeros((NVEL,) + phi.shape[-3:])
    g[0] = phi.reshape(phi.shape[-3:])
    return g


def lb2_steps(state, fe, mobility, cp, nsteps):
    """Advance an Lb2State by nsteps of the main loop with ndist = 2."""
    s = state
    L = lib()
    L.orc_lb2_step.argtypes = [_I3, ctypes.POINTER(SymmParam),
                               ctypes.c_double, ctypes.POINTER(CollideParam),
                               _P, _P, _P, _P, _P, _P, ctypes.c_int]
    L.orc_lb2_step(_dims(s.L), ctypes.byref(fe), float(mobility),
                   ctypes.byref(cp), _p(s.f), _p(s.g), _p(s._scratch),
                   _p(s.phi), _p(s.u), _p(s._work), int(nsteps))
    return s


def collide_binary(L, fe, cp, mobility, f, g, phi):
    """One binary collision (gradients of phi computed here): (f, g, u)."""
    Lb = lib()
    Lb.orc_collide_binary.argtypes = [_I3, ctypes.POINTER(SymmParam),
                                      ctypes.POINTER(CollideParam),
                                      ctypes.c_double, _P, _P, _P, _P, _P,
                                      _P]
    f = np.ascontiguousarray(f, dtype=np.float64).copy()
    g = np.ascontiguousarray(g, dtype=np.float64).copy()
    phi = np.ascontiguousarray(phi, dtype=np.float64)
    grad, delsq = grad_7pt(L, phi)
    u = np.zeros((3,) + tuple(L))
    Lb.orc_collide_binary(_dims(L), ctypes.byref(fe), ctypes.byref(cp),
                          float(mobility), _p(f), _p(g), _p(phi), _p(grad),
                          _p(delsq), _p(u))
    return f, g, u


def field_stats(L, q):
    out = np.zeros(5)
    lib().orc_field_stats(_dims(L), _p(np.ascontiguousarray(q[0] if q.ndim == 4
                                                           else q)), _p(out))
    return out


def symm_fed_total(L, fe, phi):
    grad, _ = grad_7pt(L, phi)
    return lib().orc_symm_fed_total(_dims(L), ctypes.byref(fe), _p(phi),
                                    _p(grad))


# ---------------------------------------------------------------------------
# The reference itself (only where oracle/_ref was built from its sources)
# ---------------------------------------------------------------------------

def have_reference():
    return os.path.exists(REF_SHIM)


def write_arrays(prefix, **arrays):
    for name, a in arrays.items():
        np.ascontiguousarray(a, dtype=np.float64).tofile(
            "%s_%s.bin" % (prefix, name))


def read_array(prefix, name, shape):
    return np.fromfile("%s_%s.bin" % (prefix, name)).reshape(shape)


def run_reference(args, threads=1):
    """Run oracle/_ref/ref_shim with key=value arguments."""
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    out = subprocess.run([REF_SHIM] + ["%s=%s" % kv for kv in args.items()],
                         capture_output=True, text=True, env=env)
    if out.returncode != 0:
        raise RuntimeError("ref_shim failed: " + out.stderr[-2000:])
    return out.stdout


# ---------------------------------------------------------------------------
# Cholesteric liquid crystal
# ---------------------------------------------------------------------------

NQAB = 5


class LcParam(ctypes.Structure):
    _fields_ = [("a0", ctypes.c_double), ("q0", ctypes.c_double),
                ("gamma", ctypes.c_double), ("kappa0", ctypes.c_double),
                ("kappa1", ctypes.c_double), ("xi", ctypes.c_double),
                ("redshift", ctypes.c_double), ("rredshift", ctypes.c_double),
                ("epsilon", ctypes.c_double), ("e0", ctypes.c_double * 3),
                ("coswt", ctypes.c_double), ("amplitude0", ctypes.c_double)]


def lc_param(a0=0.01, gamma=3.0, kappa0=0.01, kappa1=0.01, pitch=32.0,
             xi=0.7, redshift=1.0, amplitude=-0.2):
    """As fe_lc_param_set (src/blue_phase.c:241-260); no electric field."""
    p = LcParam()
    p.a0, p.gamma, p.kappa0, p.kappa1 = a0, gamma, kappa0, kappa1
    p.q0 = 2.0 * 3.1415926535897932385 / pitch
    p.xi = xi
    p.redshift = redshift
    p.rredshift = 1.0 / redshift
    p.epsilon = 0.0
    p.coswt = 1.0
    p.amplitude0 = amplitude
    return p


def _declare_lc(L):
    LP = ctypes.POINTER(LcParam)
    L.orc_lc_mol_field.argtypes = [_I3, LP, _P, _P, _P, _P]
    L.orc_lc_stress.argtypes = [_I3, LP, _P, _P, _P, _P]
    L.orc_lc_fed.argtypes = [_I3, LP, _P, _P, _P]
    L.orc_beris_edw_update.argtypes = [_I3, LP, ctypes.c_double, _U8, _P, _P,
                                       _P, _P, _P]
    L.orc_lc_step.argtypes = [_I3, LP, ctypes.c_double,
                              ctypes.POINTER(CollideParam), _U8, _P, _P, _P,
                              _P, _P, _P, _P, ctypes.c_int]
    L.orc_lc_init_o8m.argtypes = [_I3, LP, _P]


def lc_lib():
    L = lib()
    if not getattr(L, "_lc_declared", False):
        _declare_lc(L)
        L._lc_declared = True
    return L


def lc_init_o8m(L, p):
    q = np.zeros((NQAB,) + tuple(L))
    lc_lib().orc_lc_init_o8m(_dims(L), ctypes.byref(p), _p(q))
    return q


def lc_fields(L, p, q):
    """(h[5], stress[9], fed[1]) of a given q."""
    q = np.ascontiguousarray(q, dtype=np.float64)
    grad, delsq = grad_7pt(L, q)
    h = np.zeros((NQAB,) + tuple(L))
    s = np.zeros((9,) + tuple(L))
    fed = np.zeros((1,) + tuple(L))
    Lb = lc_lib()
    Lb.orc_lc_mol_field(_dims(L), ctypes.byref(p), _p(q), _p(grad), _p(delsq),
                        _p(h))
    Lb.orc_lc_stress(_dims(L), ctypes.byref(p), _p(q), _p(grad), _p(delsq),
                     _p(s))
    Lb.orc_lc_fed(_dims(L), ctypes.byref(p), _p(q), _p(grad), _p(fed))
    return h, s, fed


def lc_be_update(L, p, gamma_rot, q, u, status=None):
    q = np.ascontiguousarray(q, dtype=np.float64).copy()
    u = np.ascontiguousarray(u, dtype=np.float64)
    grad, delsq = grad_7pt(L, q)
    work = np.zeros((30,) + tuple(L))
    lc_lib().orc_beris_edw_update(_dims(L), ctypes.byref(p), float(gamma_rot),
                                  _u8(status), _p(u), _p(grad), _p(delsq),
                                  _p(q), _p(work))
    return q


class LcState:
    def __init__(self, L, f, q, u=None):
        self.L = tuple(int(v) for v in L)
        n = self.L
        self.f = np.ascontiguousarray(f, dtype=np.float64).copy()
        self.q = np.ascontiguousarray(q, dtype=np.float64).copy()
        self.u = (np.zeros((3,) + n) if u is None else
                  np.ascontiguousarray(u, dtype=np.float64).copy())
        self.rho = np.zeros((1,) + n)
        self.force = np.zeros((3,) + n)
        self._fs = np.zeros_like(self.f)
        self._work = np.zeros((50,) + n)


def lc_steps(state, p, gamma_rot, cp, nsteps, status=None):
    s = state
    lc_lib().orc_lc_step(_dims(s.L), ctypes.byref(p), float(gamma_rot),
                         ctypes.byref(cp), _u8(status), _p(s.f), _p(s._fs),
                         _p(s.q), _p(s.u), _p(s.rho), _p(s.force),
                         _p(s._work), int(nsteps))
    return s


# ---------------------------------------------------------------------------
# Domain length from the structure factor, util/length_from_sk.c:88-190
# ---------------------------------------------------------------------------

NBIN = 128


def _wavevectors_reference(n, nref):
    """k_i of util/length_from_sk.c:126-139 in its own arithmetic: FP32,
    kmax = float(4 atan 1), dk = float(2 kmax / nref) (nref = the x extent,
    the program assumes a cube), kx = dk*i, and kx -= kmax for i > n/2."""
    f32 = np.float32
    kmax = f32(4.0 * np.arctan(1.0))
    dk = f32(2.0 * np.float64(kmax) / nref)
    i = np.arange(n)
    k = (dk * i.astype(f32)).astype(f32)
    return np.where(i > n // 2, (k - kmax).astype(f32), k).astype(f32), kmax


def structure_factor(phi, faithful=True):
    """Binned |phi(k)|^2 sums and counts over the half space k_z >= 0.

    faithful=True is the reference's program (util/length_from_sk.c:111-
    166): its wavevector for i > N/2 is dk*i - pi (:138), and the
    wavevectors and |k| are FP32, |k| = float(sqrt(double(kx kx + ky ky +
    kz kz))) with the products and sums rounded to FP32 one by one; the
    bin is floor(|k| 128 / (sqrt(3) kmax)) in double.  The transform and the
    sums here are FP64 (the reference sums in FP32).
    faithful=False uses dk*i - 2 pi and FP64 throughout.
    """
    phi = np.asarray(phi, dtype=np.float64)
    if phi.ndim == 4:
        phi = phi[0]
    nx, ny, nz = phi.shape
    c = np.fft.fftn(phi)
    if faithful:
        f32 = np.float32
        kx, kmax = _wavevectors_reference(nx, nx)
        ky, _ = _wavevectors_reference(ny, nx)
        kz = _wavevectors_reference(nz, nx)[0][:nz // 2 + 1]
        KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing="ij")
        s2 = ((KX * KX).astype(f32) + (KY * KY).astype(f32)).astype(f32)
        s2 = (s2 + (KZ * KZ).astype(f32)).astype(f32)
        kmod = np.sqrt(s2.astype(np.float64)).astype(f32)
        n = np.floor(kmod.astype(np.float64) * NBIN
                     / (np.sqrt(3.0) * np.float64(kmax))).astype(int)
    else:
        kx = 2.0 * np.pi * np.arange(nx) / nx
        kx = np.where(np.arange(nx) > nx // 2, kx - 2.0 * np.pi, kx)
        ky = 2.0 * np.pi * np.arange(ny) / ny
        ky = np.where(np.arange(ny) > ny // 2, ky - 2.0 * np.pi, ky)
        kz = 2.0 * np.pi * np.arange(nz // 2 + 1) / nz
        KX, KY, KZ = np.meshgrid(kx, ky, kz, indexing="ij")
        kmod = np.sqrt(KX * KX + KY * KY + KZ * KZ)
        n = np.floor(kmod * NBIN / (np.sqrt(3.0) * np.pi)).astype(int)
    n = np.minimum(n, NBIN - 1)
    s = np.abs(c[:, :, :nz // 2 + 1]) ** 2
    sk = np.bincount(n.ravel(), weights=s.ravel(), minlength=NBIN)
    nk = np.bincount(n.ravel(), minlength=NBIN).astype(np.float64)
    return sk, nk


def length_from_sk(phi, faithful=True):
    """L = 2 pi sum S dk / sum k S dk (util/length_from_sk.c:170-185)."""
    sk, nk = structure_factor(phi, faithful)
    dk = np.sqrt(3.0) * np.pi / NBIN
    sbar = np.where(nk != 0, sk / np.where(nk == 0, 1, nk), 0.0)
    kk = (np.arange(NBIN) + 0.5) * dk
    return 2.0 * np.pi * np.sum(dk * sbar) / np.sum(kk * dk * sbar)


# ---------------------------------------------------------------------------
# Learned corrector: double-precision restatement of the network
# (cnn_oracle.c).  No reference counterpart: checked by finite differences.
# ---------------------------------------------------------------------------

CNN_C = 32
CNN_NTAP = 27
CNN_WL = CNN_NTAP * CNN_C * CNN_C
CNN_PL = CNN_WL + CNN_C
CNN_NLAYER = 4
_F32 = ctypes.POINTER(ctypes.c_float)


def _cnn_lib():
    L = lib()
    if not getattr(L, "_cnn_declared", False):
        L.orc_cnn_forward.argtypes = [_I3, ctypes.c_int, _F32, _F32, _F32,
                                      _F32, _P]
        L.orc_cnn_loss_grad.argtypes = [_I3, ctypes.c_int, _F32, _F32, _F32,
                                        _F32, _F32, _P, _P, _P]
        L.orc_conv3_fwd.argtypes = [_I3, _P, _P, _P, _P]
        L.orc_conv3_bwd_data.argtypes = [_I3, _P, _P, _P]
        L.orc_conv3_wgrad.argtypes = [_I3, _P, _P, _P, _P]
        L.orc_bf16_round.argtypes = [ctypes.c_double]
        L.orc_bf16_round.restype = ctypes.c_double
        L._cnn_declared = True
    return L


def _f32(a):
    a = np.ascontiguousarray(a, dtype=np.float32)
    return a, a.ctypes.data_as(_F32)


def _f64(a):
    a = np.ascontiguousarray(a, dtype=np.float64)
    return a, a.ctypes.data_as(_P)


def bf16_round(a):
    """Round to bfloat16 (nearest even) and back, elementwise (numpy)."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def cnn_split(params):
    """Flat parameters -> (W [4,27,32,32], b [4,32]) views."""
    p = np.asarray(params, dtype=np.float32).reshape(CNN_NLAYER, CNN_PL)
    return (p[:, :CNN_WL].reshape(CNN_NLAYER, CNN_NTAP, CNN_C, CNN_C),
            p[:, CNN_WL:])


def cnn_forward(n, in5, scale, params, emulate=True):
    """Network output [4, N] for inputs in5 [5, N] (features in5 * scale)."""
    L = _cnn_lib()
    N = n[0] * n[1] * n[2]
    W, b = cnn_split(params)
    i5, pi5 = _f32(in5)
    sc, psc = _f32(scale)
    w, pw = _f32(W)
    bb, pb = _f32(b)
    out = np.zeros((4, N))
    rc = L.orc_cnn_forward(_I3(*n), int(emulate), pi5, psc, pw, pb,
                           out.ctypes.data_as(_P))
    assert rc == 0
    return out


def cnn_loss_grad(n, in5, scale, t4, params, emulate=True):
    """(loss, gradient as a flat [4*(27*1024+32)] array)."""
    L = _cnn_lib()
    W, b = cnn_split(params)
    i5, pi5 = _f32(in5)
    sc, psc = _f32(scale)
    t, pt = _f32(t4)
    w, pw = _f32(W)
    bb, pb = _f32(b)
    loss = ctypes.c_double()
    dW = np.zeros((CNN_NLAYER, CNN_WL))
    db = np.zeros((CNN_NLAYER, CNN_C))
    rc = L.orc_cnn_loss_grad(_I3(*n), int(emulate), pi5, psc, pt, pw, pb,
                             ctypes.byref(loss), dW.ctypes.data_as(_P),
                             db.ctypes.data_as(_P))
    assert rc == 0
    return loss.value, np.concatenate([dW, db], axis=1).ravel()


def conv3_fwd(n, a, w, b):
    """z[s][n] = b[n] + sum_t sum_c a[s+e_t][c] w[t][n][c] (double)."""
    L = _cnn_lib()
    N = n[0] * n[1] * n[2]
    a, pa = _f64(a)
    w, pw = _f64(w)
    b, pb = _f64(np.zeros(CNN_C) if b is None else b)
    z = np.zeros((N, CNN_C))
    L.orc_conv3_fwd(_I3(*n), pa, pw, pb, z.ctypes.data_as(_P))
    return z


def conv3_bwd_data(n, g, w):
    """da[s][c] = sum_t sum_o g[s-e_t][o] w[t][o][c] (double)."""
    L = _cnn_lib()
    N = n[0] * n[1] * n[2]
    g, pg = _f64(g)
    w, pw = _f64(w)
    da = np.zeros((N, CNN_C))
    L.orc_conv3_bwd_data(_I3(*n), pg, pw, da.ctypes.data_as(_P))
    return da


def conv3_wgrad(n, g, a):
    """(dw[t][o][c] = sum_s g[s-e_t][o] a[s][c], db[o] = sum_s g[s][o])."""
    L = _cnn_lib()
    g, pg = _f64(g)
    a, pa = _f64(a)
    dw = np.zeros((CNN_NTAP, CNN_C, CNN_C))
    db = np.zeros(CNN_C)
    L.orc_conv3_wgrad(_I3(*n), pg, pa, dw.ctypes.data_as(_P),
                      db.ctypes.data_as(_P))
    return dw, db


# ---------------------------------------------------------------------------
# Snapshot files (restatement of the reference's file format)
# ---------------------------------------------------------------------------

def _metadata_json(L, fmt, count):
    """The JSON of io_metadata_to_json (src/io_metadata.c:159) as cJSON
    prints it, for one rank and one file."""
    b = fmt == "binary"
    t = "\t"
    lines = [
        "{",
        t + '"coords":' + t + "{",
        t * 2 + '"options":' + t + "{",
        t * 3 + '"System size (total)":' + t + "[%d, %d, %d]," % tuple(L),
        t * 3 + '"Periodic boundaries":' + t + "[1, 1, 1],",
        t * 3 + '"Left-end limit Lmin":' + t + "[0.5, 0.5, 0.5]",
        t * 2 + "},",
        t * 2 + '"lees_edwards":' + t + "{",
        t * 3 + '"Number of planes":' + t + "0",
        t * 2 + "}",
        t + "},",
        t + '"io_options":' + t + "{",
        t * 2 + '"Mode":' + t + '"mpiio",',
        t * 2 + '"Record format":' + t + '"%s",' % fmt,
        t * 2 + '"Metadata version":' + t + "3,",
        t * 2 + '"Report":' + t + "false,",
        t * 2 + '"Asynchronous":' + t + "false,",
        t * 2 + '"Compression level":' + t + "0,",
        t * 2 + '"I/O grid":' + t + "[1, 1, 1]",
        t + "},",
        t + '"io_element":' + t + "{",
        t * 2 + '"MPI_Datatype":' + t + ('"MPI_DOUBLE",' if b
                                         else '"MPI_CHAR",'),
        t * 2 + '"Size (bytes)":' + t + ("8," if b else "1,"),
        t * 2 + '"Count":' + t + "%d," % count,
        t * 2 + '"Endianness":' + t + '"LITTLE_ENDIAN"',
        t + "},",
        t + '"io_subfile":' + t + "{",
        t * 2 + '"Number of files":' + t + "1,",
        t * 2 + '"File index":' + t + "0,",
        t * 2 + '"Topology":' + t + "[1, 1, 1],",
        t * 2 + '"Coordinate":' + t + "[0, 0, 0],",
        t * 2 + '"Data ndims":' + t + "3,",
        t * 2 + '"File size (sites)":' + t + "[%d, %d, %d]," % tuple(L),
        t * 2 + '"File offset (sites)":' + t + "[0, 0, 0]",
        t + "}",
        "}"]
    return "\n".join(lines).encode()


def snapshot_files(L, step, f=None, ndist=1, fields=None, fmt="binary"):
    """{file name: bytes} of lb_io_write (src/lb_data.c:1716, records of
    lb_write_buf(_ascii) :1533-1610) and field_io_write (src/field.c:1633,
    records of field_write_buf(_ascii) :896-965; hydro_io_write,
    src/hydro.c:941, writes the fields "rho" and "vel") for
    component-major arrays f [ndist*19, L] and fields {name: [nf, L]}:
    sites in x, y, z order."""
    out = {}
    n = L[0] * L[1] * L[2]

    def records(a, nrow, ncol):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(ncol, nrow, n)
        if fmt == "binary":
            # record: value (col, row) at col*nrow + row
            return np.ascontiguousarray(
                a.transpose(2, 0, 1)).astype("<f8").tobytes()
        buf = []
        for i in range(n):
            for r in range(nrow):
                buf.append("".join(" %22.15e" % a[c, r, i]
                                   for c in range(ncol)) + "\n")
        return "".join(buf).encode()

    if f is not None:
        cnt = ndist * 19 if fmt == "binary" else 19 * (ndist * 23 + 1)
        out["dist-metadata.001-001"] = _metadata_json(L, fmt, cnt)
        out["dist-%09d.001-001" % step] = records(f, 19, ndist)
    for stub, a in (fields or {}).items():
        nf = a.shape[0]
        cnt = nf if fmt == "binary" else nf * 23 + 1
        out["%s-metadata.001-001" % stub] = _metadata_json(L, fmt, cnt)
        out["%s-%09d.001-001" % (stub, step)] = records(a, 1, nf)
    return out

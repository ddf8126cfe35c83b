"""ludwig_gb300: the Ludwig lattice-Boltzmann time step on one GB300.

Python mirror of the C ABI in ``include/ludwig_gb.h`` (ctypes over the
in-tree ``libludwig_gb.so``).  Objects carry the reference's names
(``cs_t`` -> :class:`Coords`, ``lb_t`` -> :class:`LB`, ``field_t`` ->
:class:`Field`, ...) and their methods call the C entry points of the same
name.  There is no CPU fallback: if the CUDA library is missing or no GPU is
visible, loading fails with an error.

Host arrays use the layout of the C ABI: numpy float64, shape
``(ncomp, Lx, Ly, Lz)``, C order.
"""

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libludwig_gb.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "ludwig_gb.h")

FP64, FP32, FP16 = 0, 1, 2
NVEL = 19

_lib = None


class LudwigGBError(RuntimeError):
    pass


def build(verbose=False, force=False):
    from . import buildlib
    return buildlib.build(verbose=verbose, force=force)


def load_library(path=LIB_PATH):
    """Load libludwig_gb.so (no GPU needed to load)."""
    global _lib
    if _lib is None:
        if not os.path.exists(path):
            raise LudwigGBError(
                "libludwig_gb.so is not built (run ludwig_gb300.build())")
        _lib = ctypes.CDLL(path)
        _declare(_lib)
    return _lib


_P = ctypes.c_void_p
_D = ctypes.POINTER(ctypes.c_double)
_I3 = ctypes.c_int * 3
_D3 = ctypes.c_double * 3
_IORF = {"ascii": 1, "binary": 2}          # enum io_record_format_enum
_F = ctypes.POINTER(ctypes.c_float)


class IoOptions(ctypes.Structure):
    """io_options_t (src/io_options.h:46-54)"""
    _fields_ = [("mode", ctypes.c_int), ("iorformat", ctypes.c_int),
                ("metadata_version", ctypes.c_int), ("report", ctypes.c_int),
                ("asynchronous", ctypes.c_int),
                ("compression_levl", ctypes.c_int),
                ("iogrid", ctypes.c_int * 3)]


class IoInfoArgs(ctypes.Structure):
    """io_info_args_t (src/io_info_args.h:33-38)"""
    _fields_ = [("input", IoOptions), ("output", IoOptions),
                ("grid", ctypes.c_int * 3), ("iofreq", ctypes.c_int)]


class LbDataOptions(ctypes.Structure):
    """lb_data_options_t (src/lb_data_options.h:32-42)"""
    _fields_ = [("ndim", ctypes.c_int), ("nvel", ctypes.c_int),
                ("ndist", ctypes.c_int), ("nrelax", ctypes.c_int),
                ("halo", ctypes.c_int), ("reportimbalance", ctypes.c_int),
                ("usefirsttouch", ctypes.c_int), ("iodata", IoInfoArgs)]


class FieldOptions(ctypes.Structure):
    """field_options_t (src/field_options.h:28-37)"""
    _fields_ = [("ndata", ctypes.c_int), ("nhcomm", ctypes.c_int),
                ("haloscheme", ctypes.c_int), ("haloverbose", ctypes.c_int),
                ("usefirsttouch", ctypes.c_int), ("iodata", IoInfoArgs)]


class HydroOptions(ctypes.Structure):
    """hydro_options_t (src/hydro_options.h:22-30)"""
    _fields_ = [("nhcomm", ctypes.c_int), ("rho", FieldOptions),
                ("u", FieldOptions), ("force", FieldOptions),
                ("eta", FieldOptions)]


class MapOptions(ctypes.Structure):
    """map_options_t (src/map_options.h:21-26)"""
    _fields_ = [("ndata", ctypes.c_int), ("is_porous_media", ctypes.c_int),
                ("filestub", ctypes.c_char_p), ("iodata", IoInfoArgs)]


class FeSymmParam(ctypes.Structure):
    _fields_ = [("a", ctypes.c_double), ("b", ctypes.c_double),
                ("kappa", ctypes.c_double), ("c", ctypes.c_double),
                ("h", ctypes.c_double)]


class PhiChInfo(ctypes.Structure):
    _fields_ = [("conserve", ctypes.c_int), ("noise", ctypes.c_int)]


class BoxParam(ctypes.Structure):
    _fields_ = [("ntotal", ctypes.c_int * 3), ("rho0", ctypes.c_double),
                ("eta", ctypes.c_double), ("eta_bulk", ctypes.c_double),
                ("a", ctypes.c_double), ("b", ctypes.c_double),
                ("kappa", ctypes.c_double), ("mobility", ctypes.c_double),
                ("seed", ctypes.c_int), ("phi0", ctypes.c_double),
                ("noise", ctypes.c_double)]


class LcAnchoringParam(ctypes.Structure):
    """lc_anchoring_param_t (src/lc_anchoring.h:30-35)"""
    _fields_ = [("type", ctypes.c_int), ("w1", ctypes.c_double),
                ("w2", ctypes.c_double), ("nfix", ctypes.c_double * 3)]


class FeLcParam(ctypes.Structure):
    _fields_ = [("a0", ctypes.c_double), ("q0", ctypes.c_double),
                ("gamma", ctypes.c_double), ("kappa0", ctypes.c_double),
                ("kappa1", ctypes.c_double), ("xi", ctypes.c_double),
                ("zeta0", ctypes.c_double), ("zeta1", ctypes.c_double),
                ("zeta2", ctypes.c_double), ("redshift", ctypes.c_double),
                ("rredshift", ctypes.c_double), ("epsilon", ctypes.c_double),
                ("amplitude0", ctypes.c_double), ("e0", ctypes.c_double * 3),
                ("coswt", ctypes.c_double),
                ("is_redshift_updated", ctypes.c_int),
                ("is_active", ctypes.c_int),
                ("coll", LcAnchoringParam), ("wall", LcAnchoringParam)]


class BerisEdwParam(ctypes.Structure):
    _fields_ = [("xi", ctypes.c_double), ("gamma", ctypes.c_double),
                ("noise", ctypes.c_int), ("var", ctypes.c_double),
                ("tmatrix", ctypes.c_double * 45)]


def _declare(L):
    pp = ctypes.POINTER(ctypes.c_void_p)
    sig = {
        "ludwig_gb_last_error": ([], ctypes.c_char_p),
        "ludwig_gb_version": ([], ctypes.c_char_p),
        "ludwig_gb_stream": ([], _P),
        "ludwig_gb_sync": ([], ctypes.c_int),
        "ludwig_gb_tune_set": ([ctypes.c_int] * 3, ctypes.c_int),
        "ludwig_gb_tune_sites": ([ctypes.c_int], ctypes.c_int),
        "ludwig_gb_selftest_bounded_wait": ([_D], ctypes.c_int),
        "ludwig_gb_lb_fp16_rescale": ([_P, _D], ctypes.c_int),
        "pe_create": ([ctypes.c_int, pp], ctypes.c_int),
        "pe_free": ([_P], ctypes.c_int),
        "cs_create": ([_P, pp], ctypes.c_int),
        "cs_free": ([_P], ctypes.c_int),
        "cs_ntotal_set": ([_P, _I3], ctypes.c_int),
        "cs_nhalo_set": ([_P, ctypes.c_int], ctypes.c_int),
        "cs_init": ([_P], ctypes.c_int),
        "physics_create": ([_P, pp], ctypes.c_int),
        "physics_free": ([_P], ctypes.c_int),
        "physics_rho0_set": ([_P, ctypes.c_double], ctypes.c_int),
        "physics_eta_shear_set": ([_P, ctypes.c_double], ctypes.c_int),
        "physics_eta_bulk_set": ([_P, ctypes.c_double], ctypes.c_int),
        "physics_mobility_set": ([_P, ctypes.c_double], ctypes.c_int),
        "physics_fbody_set": ([_P, _D3], ctypes.c_int),
        "physics_e0_frequency_set": ([_P, ctypes.c_double], ctypes.c_int),
        "physics_control_init_time": ([_P, ctypes.c_int, ctypes.c_int],
                                      ctypes.c_int),
        "physics_control_next_step": ([_P], ctypes.c_int),
        "physics_control_timestep": ([_P], ctypes.c_int),
        "physics_control_time": ([_P, _D], ctypes.c_int),
        "lb_data_create": ([_P, _P, ctypes.POINTER(LbDataOptions), pp],
                           ctypes.c_int),
        "ludwig_gb_lb_data_create": ([_P, _P, ctypes.POINTER(LbDataOptions),
                                      ctypes.c_int, ctypes.c_double, pp],
                                     ctypes.c_int),
        "lb_data_options_default": ([], LbDataOptions),
        "lb_data_options_ndim_nvel_ndist": ([ctypes.c_int] * 3, LbDataOptions),
        "field_options_default": ([], FieldOptions),
        "field_options_ndata_nhalo": ([ctypes.c_int] * 2, FieldOptions),
        "hydro_options_default": ([], HydroOptions),
        "hydro_options_nhalo": ([ctypes.c_int], HydroOptions),
        "map_options_default": ([], MapOptions),
        "map_options_ndata": ([ctypes.c_int], MapOptions),
        "io_options_default": ([], IoOptions),
        "io_info_args_default": ([], IoInfoArgs),
        "ludwig_gb_field_create": ([_P, _P, _P, ctypes.c_char_p,
                                    ctypes.POINTER(FieldOptions), ctypes.c_int,
                                    pp], ctypes.c_int),
        "ludwig_gb_hydro_create": ([_P, _P, _P, ctypes.POINTER(HydroOptions),
                                    ctypes.c_int, pp], ctypes.c_int),
        "cs_index": ([_P, ctypes.c_int, ctypes.c_int, ctypes.c_int],
                     ctypes.c_int),
        "cs_nsites": ([_P, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "cs_nhalo": ([_P, ctypes.POINTER(ctypes.c_int)], ctypes.c_int),
        "cs_strides": ([_P] + [ctypes.POINTER(ctypes.c_int)] * 3,
                       ctypes.c_int),
        "cs_index_to_ijk": ([_P, ctypes.c_int, ctypes.POINTER(ctypes.c_int)],
                            ctypes.c_int),
        "field_scalar": ([_P, ctypes.c_int, _D], ctypes.c_int),
        "field_scalar_set": ([_P, ctypes.c_int, ctypes.c_double],
                             ctypes.c_int),
        "field_tensor": ([_P, ctypes.c_int, _D], ctypes.c_int),
        "field_scalar_array": ([_P, ctypes.c_int, _D], ctypes.c_int),
        "ludwig_gb_lb_to_host_cs": ([_P, ctypes.c_int, _D], ctypes.c_int),
        "ludwig_gb_lb_from_host_cs": ([_P, ctypes.c_int, _D], ctypes.c_int),
        "ludwig_gb_field_to_host_cs": ([_P, ctypes.c_int, _D], ctypes.c_int),
        "ludwig_gb_field_from_host_cs": ([_P, ctypes.c_int, _D],
                                         ctypes.c_int),
        "ludwig_gb_hydro_to_host_cs": ([_P, ctypes.c_int, _D, _D, _D],
                                       ctypes.c_int),
        "lb_free": ([_P], ctypes.c_int),
        "lb_init_rest_f": ([_P, ctypes.c_double], ctypes.c_int),
        "lb_halo": ([_P], ctypes.c_int),
        "lb_f_to_host": ([_P, _D], ctypes.c_int),
        "lb_io_record_format_set": ([_P, ctypes.c_int, ctypes.c_int],
                                    ctypes.c_int),
        "field_io_record_format_set": ([_P, ctypes.c_int, ctypes.c_int],
                                       ctypes.c_int),
        "lb_io_write": ([_P, ctypes.c_int, _P], ctypes.c_int),
        "lb_io_read": ([_P, ctypes.c_int, _P], ctypes.c_int),
        "field_io_write": ([_P, ctypes.c_int, _P], ctypes.c_int),
        "field_io_read": ([_P, ctypes.c_int, _P], ctypes.c_int),
        "hydro_io_record_format_set": ([_P, ctypes.c_int, ctypes.c_int],
                                       ctypes.c_int),
        "hydro_io_write": ([_P, ctypes.c_int, _P], ctypes.c_int),
        "hydro_io_read": ([_P, ctypes.c_int, _P], ctypes.c_int),
        "lb_f_from_host": ([_P, _D], ctypes.c_int),
        "lb_collide": ([_P, _P, _P, _P, _P, _P], ctypes.c_int),
        "lb_g_to_host": ([_P, _D], ctypes.c_int),
        "lb_g_from_host": ([_P, _D], ctypes.c_int),
        "phi_lb_to_field": ([_P, _P], ctypes.c_int),
        "phi_lb_from_field": ([_P, _P], ctypes.c_int),
        "ludwig_gb_lb2_step": ([_P] * 4 + [ctypes.c_int], ctypes.c_int),
        "lb_propagation": ([_P], ctypes.c_int),
        "field_create": ([_P, _P, _P, ctypes.c_char_p,
                          ctypes.POINTER(FieldOptions), pp], ctypes.c_int),
        "field_free": ([_P], ctypes.c_int),
        "field_halo": ([_P], ctypes.c_int),
        "field_to_host": ([_P, _D], ctypes.c_int),
        "field_from_host": ([_P, _D], ctypes.c_int),
        "field_phi_init_spinodal": ([_P, ctypes.c_int, ctypes.c_double,
                                     ctypes.c_double], ctypes.c_int),
        "field_phi_init_spinodal_patches": ([_P, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_double], ctypes.c_int),
        "field_phi_init_drop": ([_P] + [ctypes.c_double] * 3 + [ctypes.c_int],
                                ctypes.c_int),
        "field_grad_create": ([_P, _P, ctypes.c_int, pp], ctypes.c_int),
        "field_grad_free": ([_P], None),
        "field_grad_compute": ([_P], ctypes.c_int),
        "field_grad_stencil_set": ([_P, ctypes.c_int], ctypes.c_int),
        "advection_order_set": ([ctypes.c_int], ctypes.c_int),
        "field_grad_to_host": ([_P, _D, _D], ctypes.c_int),
        "hydro_create": ([_P, _P, _P, ctypes.POINTER(HydroOptions), pp],
                         ctypes.c_int),
        "hydro_free": ([_P], ctypes.c_int),
        "hydro_f_zero": ([_P, _D3], ctypes.c_int),
        "hydro_u_zero": ([_P, _D3], ctypes.c_int),
        "hydro_u_halo": ([_P], ctypes.c_int),
        "hydro_to_host": ([_P, _D, _D, _D], ctypes.c_int),
        "hydro_from_host": ([_P, _D, _D, _D], ctypes.c_int),
        "map_create": ([_P, _P, ctypes.POINTER(MapOptions), pp],
                       ctypes.c_int),
        "map_free": ([pp], ctypes.c_int),
        "map_status_from_host": ([_P, ctypes.POINTER(ctypes.c_uint8)],
                                 ctypes.c_int),
        "fe_symm_create": ([_P, _P, _P, _P, pp], ctypes.c_int),
        "fe_symm_free": ([_P], ctypes.c_int),
        "fe_symm_param_set": ([_P, FeSymmParam], ctypes.c_int),
        "pth_create": ([_P, _P, ctypes.c_int, pp], ctypes.c_int),
        "pth_free": ([_P], ctypes.c_int),
        "pth_stress_compute": ([_P, _P], ctypes.c_int),
        "pth_to_host": ([_P, _D], ctypes.c_int),
        "phi_force_calculation": ([_P] * 9, ctypes.c_int),
        "phi_ch_create": ([_P, _P, _P, ctypes.POINTER(PhiChInfo), pp],
                          ctypes.c_int),
        "phi_ch_free": ([_P], ctypes.c_int),
        "phi_cahn_hilliard": ([_P] * 6, ctypes.c_int),
        "ludwig_gb_binary_step": ([_P] * 5 + [ctypes.c_int], ctypes.c_int),
        "ludwig_gb_binary_step_async": ([_P] * 5 + [ctypes.c_int],
                                        ctypes.c_int),
        "ludwig_gb_state_bytes": ([_P] + [ctypes.POINTER(ctypes.c_size_t)]
                                  * 3, ctypes.c_int),
        "ludwig_gb_state_to_host_async": ([_P] * 6, ctypes.c_int),
        "ludwig_gb_state_from_host_async": ([_P] * 6, ctypes.c_int),
        "ludwig_gb_host_alloc": ([ctypes.c_size_t, pp], ctypes.c_int),
        "ludwig_gb_host_free": ([_P], ctypes.c_int),
        "ludwig_gb_time_binary": ([_P] * 5 + [ctypes.c_int, _D],
                                  ctypes.c_int),
        "ludwig_gb_time_binary_e2e": ([_P] * 5 + [ctypes.c_int] + [_P] * 4
                                      + [_D], ctypes.c_int),
        "ludwig_gb_time_binary_e2e_overlap": ([_P] * 5 + [ctypes.c_int]
                                              + [_P] * 7 + [_D],
                                              ctypes.c_int),
        "fe_lc_create": ([_P, _P, _P, _P, _P, pp], ctypes.c_int),
        "fe_lc_free": ([_P], ctypes.c_int),
        "fe_lc_param_set": ([_P, ctypes.POINTER(FeLcParam)], ctypes.c_int),
        "blue_phase_O8M_init": ([_P, ctypes.POINTER(FeLcParam), _P, _D],
                                ctypes.c_int),
        "blue_phase_O2_init": ([_P, ctypes.POINTER(FeLcParam), _P, _D],
                               ctypes.c_int),
        "blue_phase_nematic_init": ([_P, ctypes.POINTER(FeLcParam), _P, _D],
                                    ctypes.c_int),
        "blue_phase_random_q_init": ([_P, ctypes.POINTER(FeLcParam), _P],
                                     ctypes.c_int),
        "blue_phase_twist_init": ([_P, ctypes.POINTER(FeLcParam), _P,
                                   ctypes.c_int], ctypes.c_int),
        "blue_phase_random_q_rectangle": ([_P, ctypes.POINTER(FeLcParam), _P,
                                           ctypes.POINTER(ctypes.c_int),
                                           ctypes.POINTER(ctypes.c_int)],
                                          ctypes.c_int),
        "beris_edw_create": ([_P, _P, _P, pp], ctypes.c_int),
        "beris_edw_free": ([_P], ctypes.c_int),
        "beris_edw_param_set": ([_P, ctypes.POINTER(BerisEdwParam)],
                                ctypes.c_int),
        "beris_edw_update": ([_P] * 8, ctypes.c_int),
        "beris_edw_h_to_host": ([_P, _D], ctypes.c_int),
        "ludwig_gb_lc_step": ([_P] * 6 + [ctypes.c_int], ctypes.c_int),
        "ludwig_gb_time_lc": ([_P] * 6 + [ctypes.c_int, _D], ctypes.c_int),
        "ludwig_gb_length_from_sk": ([_P, ctypes.c_int, _D, _D, _D],
                                     ctypes.c_int),
        "ludwig_gb_ensemble_create": ([ctypes.c_int, ctypes.POINTER(BoxParam),
                                       ctypes.c_int, pp], ctypes.c_int),
        "ludwig_gb_ensemble_free": ([_P], ctypes.c_int),
        "ludwig_gb_ensemble_step": ([_P, ctypes.c_int], ctypes.c_int),
        "ludwig_gb_ensemble_time": ([_P, ctypes.c_int, _D], ctypes.c_int),
        "ludwig_gb_ensemble_tune_set": ([_P] + [ctypes.c_int] * 3,
                                        ctypes.c_int),
        "ludwig_gb_ensemble_autotune": ([_P, ctypes.c_int,
                                         ctypes.POINTER(ctypes.c_int), _D],
                                        ctypes.c_int),
        "ludwig_gb_ensemble_box_get": ([_P, ctypes.c_int, _D, _D, _D, _D],
                                       ctypes.c_int),
        "ludwig_gb_ensemble_box_set_phi": ([_P, ctypes.c_int, _D],
                                           ctypes.c_int),
        "ludwig_gb_ensemble_check": ([_P, ctypes.POINTER(ctypes.c_int)],
                                     ctypes.c_int),
        "ludwig_gb_ensemble_box_active": ([_P, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_int)],
                                          ctypes.c_int),
        "ludwig_gb_ensemble_sites": ([_P, ctypes.POINTER(ctypes.c_longlong)],
                                     ctypes.c_int),
        "ludwig_gb_physics_use": ([_P], ctypes.c_int),
        "ludwig_gb_cnn_create": ([_I3, ctypes.c_ulonglong, pp], ctypes.c_int),
        "ludwig_gb_cnn_free": ([_P], ctypes.c_int),
        "ludwig_gb_cnn_nparams": ([], ctypes.c_int),
        "ludwig_gb_cnn_params_get": ([_P, _F], ctypes.c_int),
        "ludwig_gb_cnn_params_set": ([_P, _F], ctypes.c_int),
        "ludwig_gb_cnn_grads_get": ([_P, _F], ctypes.c_int),
        "ludwig_gb_cnn_scales_set": ([_P, _F, _F, _F], ctypes.c_int),
        "ludwig_gb_cnn_scales_get": ([_P, _F, _F, _F], ctypes.c_int),
        "ludwig_gb_cnn_forward": ([_P, _P, _P], ctypes.c_int),
        "ludwig_gb_cnn_forward_n": ([_P, ctypes.c_int, pp, pp], ctypes.c_int),
        "ludwig_gb_cnn_loss_grad": ([_P, _P, _P, _D], ctypes.c_int),
        "ludwig_gb_cnn_train_step": ([_P, _P, _P, ctypes.c_double, _D],
                                     ctypes.c_int),
        "ludwig_gb_cnn_train_steps": ([_P, ctypes.c_int, pp, pp,
                                       ctypes.c_double, _D], ctypes.c_int),
        "ludwig_gb_cnn_correct": ([_P] * 4, ctypes.c_int),
        "ludwig_gb_cnn_line_reuse": ([_P, ctypes.c_int], ctypes.c_int),
        "ludwig_gb_cnn_conv3": ([_P] * 4 + [ctypes.c_int, _P], ctypes.c_int),
        "ludwig_gb_cnn_wgrad3": ([_P] * 4, ctypes.c_int),
        "ludwig_gb_coarse_restrict": ([_P] * 6, ctypes.c_int),
        "ludwig_gb_fields_restrict": ([_P] * 4 + [_I3], ctypes.c_int),
        "ludwig_gb_fields_pack": ([_P] * 4, ctypes.c_int),
        "stats_field_q": ([_P, ctypes.c_int, _D], ctypes.c_int),
        "stats_distribution": ([_P, _D], ctypes.c_int),
        "stats_free_energy_symm": ([_P, _D], ctypes.c_int),
        "stats_free_energy_lc": ([_P, _D], ctypes.c_int),
        "ludwig_gb_fe_lc_stats_info": ([_P, _P, _D], ctypes.c_int),
        "ludwig_gb_stats_velocity_minmax": ([_P, _P, _D], ctypes.c_int),
    }
    for name, (args, res) in sig.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res


def lib():
    return load_library()


def _check(rc, what=""):
    if rc != 0:
        msg = lib().ludwig_gb_last_error().decode()
        raise LudwigGBError("%s failed (code %d): %s" % (what, rc, msg))


def _new(fn, *args):
    out = ctypes.c_void_p()
    _check(getattr(lib(), fn)(*args, ctypes.byref(out)), fn)
    return out


def _dp(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


# ---------------------------------------------------------------------------
# Objects
# ---------------------------------------------------------------------------

class _Obj:
    _free = None

    def __init__(self):
        self.ptr = None

    def close(self):
        if self.ptr is not None and self._free is not None:
            getattr(lib(), self._free)(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PE(_Obj):
    _free = "pe_free"

    def __init__(self, device=0):
        super().__init__()
        self.ptr = _new("pe_create", int(device))


class Coords(_Obj):
    """cs_t: periodic lattice of ntotal sites (src/coords.c)."""
    _free = "cs_free"

    def __init__(self, pe, ntotal, nhalo=2):
        super().__init__()
        self.pe = pe
        self.ntotal = tuple(int(v) for v in ntotal)
        self.ptr = _new("cs_create", pe.ptr)
        _check(lib().cs_ntotal_set(self.ptr, _I3(*self.ntotal)),
               "cs_ntotal_set")
        _check(lib().cs_nhalo_set(self.ptr, int(nhalo)), "cs_nhalo_set")
        _check(lib().cs_init(self.ptr), "cs_init")

    @property
    def nsites(self):
        return int(np.prod(self.ntotal))


class Physics(_Obj):
    _free = "physics_free"

    def __init__(self, pe, rho0=1.0, eta=1.0 / 6.0, eta_bulk=None,
                 mobility=0.0, fbody=(0.0, 0.0, 0.0)):
        super().__init__()
        self.ptr = _new("physics_create", pe.ptr)
        L = lib()
        _check(L.physics_rho0_set(self.ptr, float(rho0)), "rho0")
        _check(L.physics_eta_shear_set(self.ptr, float(eta)), "eta")
        _check(L.physics_eta_bulk_set(self.ptr, float(eta if eta_bulk is None
                                                      else eta_bulk)), "zeta")
        _check(L.physics_mobility_set(self.ptr, float(mobility)), "mobility")
        _check(L.physics_fbody_set(self.ptr, _D3(*fbody)), "fbody")


class LB(_Obj):
    """lb_t: D3Q19 distributions (src/lb_data.c)."""
    _free = "lb_free"

    def __init__(self, cs, precision=FP64, nrelax=0, fp16_scale=0.0,
                 ndist=1):
        super().__init__()
        self.cs = cs
        self.precision = precision
        self.ndist = int(ndist)
        o = lib().lb_data_options_ndim_nvel_ndist(3, 19, int(ndist))
        o.nrelax = int(nrelax)
        self.ptr = _new("ludwig_gb_lb_data_create", cs.pe.ptr, cs.ptr,
                        ctypes.byref(o), int(precision), float(fp16_scale))

    def init_rest(self, rho0=1.0):
        _check(lib().lb_init_rest_f(self.ptr, float(rho0)), "lb_init_rest_f")

    def get(self):
        f = np.zeros((NVEL,) + self.cs.ntotal)
        _check(lib().lb_f_to_host(self.ptr, _dp(f)), "lb_f_to_host")
        return f

    def set(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        assert f.shape == (NVEL,) + self.cs.ntotal
        _check(lib().lb_f_from_host(self.ptr, _dp(f)), "lb_f_from_host")

    def io_format(self, fmt_in="binary", fmt_out="binary"):
        """Record formats ("binary" or "ascii") of lb_io_read / write."""
        _check(lib().lb_io_record_format_set(self.ptr, _IORF[fmt_in],
                                             _IORF[fmt_out]), "io format")

    def io_write(self, step):
        """lb_io_write: dist-<step>.001-001 (and its metadata) in the
        current directory, in the reference's format."""
        _check(lib().lb_io_write(self.ptr, int(step), None), "lb_io_write")

    def io_read(self, step):
        _check(lib().lb_io_read(self.ptr, int(step), None), "lb_io_read")

    def get_g(self):
        """The order-parameter distribution (ndist = 2)."""
        g = np.zeros((NVEL,) + self.cs.ntotal)
        _check(lib().lb_g_to_host(self.ptr, _dp(g)), "lb_g_to_host")
        return g

    def set_g(self, g):
        g = np.ascontiguousarray(g, dtype=np.float64)
        assert g.shape == (NVEL,) + self.cs.ntotal
        _check(lib().lb_g_from_host(self.ptr, _dp(g)), "lb_g_from_host")

    def collide(self, hydro, map_=None, fe=None):
        _check(lib().lb_collide(self.ptr, hydro.ptr,
                                map_.ptr if map_ else None, None,
                                fe.ptr if fe else None, None), "lb_collide")

    def halo(self):
        _check(lib().lb_halo(self.ptr), "lb_halo")

    def propagation(self):
        _check(lib().lb_propagation(self.ptr), "lb_propagation")

    def fp16_rescale(self):
        """Derive the FP16 storage scale from the range of the stored
        deviations (returns the scale; 1 for FP32/FP64)."""
        sc = ctypes.c_double()
        _check(lib().ludwig_gb_lb_fp16_rescale(self.ptr, ctypes.byref(sc)),
               "fp16_rescale")
        return sc.value

    def moments(self):
        out = np.zeros(4)
        _check(lib().stats_distribution(self.ptr, _dp(out)),
               "stats_distribution")
        return out


class Field(_Obj):
    """field_t: nf-component site field (src/field.c)."""
    _free = "field_free"

    def __init__(self, cs, nf=1, nhalo=2, precision=FP64, name="phi"):
        super().__init__()
        self.cs = cs
        self.nf = nf
        self.name = name
        o = lib().field_options_ndata_nhalo(int(nf), int(nhalo))
        self.ptr = _new("ludwig_gb_field_create", cs.pe.ptr, cs.ptr, None,
                        name.encode(), ctypes.byref(o), int(precision))

    def get(self):
        a = np.zeros((self.nf,) + self.cs.ntotal)
        _check(lib().field_to_host(self.ptr, _dp(a)), "field_to_host")
        return a

    def set(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        assert a.shape == (self.nf,) + self.cs.ntotal
        _check(lib().field_from_host(self.ptr, _dp(a)), "field_from_host")

    def io_format(self, fmt_in="binary", fmt_out="binary"):
        """Record formats ("binary" or "ascii") of field_io_read / write."""
        _check(lib().field_io_record_format_set(self.ptr, _IORF[fmt_in],
                                                _IORF[fmt_out]), "io format")

    def io_write(self, step):
        """field_io_write: <name>-<step>.001-001 (and its metadata) in the
        current directory, in the reference's format."""
        _check(lib().field_io_write(self.ptr, int(step), None),
               "field_io_write")

    def io_read(self, step):
        _check(lib().field_io_read(self.ptr, int(step), None), "field_io_read")

    def halo(self):
        _check(lib().field_halo(self.ptr), "field_halo")

    def init_spinodal(self, seed, phi0=0.0, amp=0.02):
        _check(lib().field_phi_init_spinodal(self.ptr, int(seed), float(phi0),
                                             float(amp)), "spinodal")

    def init_patches(self, seed, patch, volminus1):
        """Cubes of patch^3 sites of -1 (probability volminus1) or +1
        (src/field_phi_init.c:537)."""
        _check(lib().field_phi_init_spinodal_patches(
            self.ptr, int(seed), int(patch), float(volminus1)), "patches")

    def init_drop(self, xi, radius, phistar=1.0, centred=False):
        """A drop of the given radius and interface width (src/
        field_phi_init.c:38)."""
        _check(lib().field_phi_init_drop(self.ptr, float(xi), float(radius),
                                         float(phistar), int(bool(centred))),
               "field_phi_init_drop")

    def length_from_sk(self, faithful=True):
        """Domain length L from the structure factor (and S, counts)."""
        L = ctypes.c_double()
        sk, nk = np.zeros(128), np.zeros(128)
        _check(lib().ludwig_gb_length_from_sk(self.ptr, int(bool(faithful)),
                                              ctypes.byref(L), _dp(sk),
                                              _dp(nk)), "length_from_sk")
        return L.value, sk, nk

    def stats(self, n=0):
        out = np.zeros(5)
        _check(lib().stats_field_q(self.ptr, int(n), _dp(out)),
               "stats_field_q")
        return out


class FieldGrad(_Obj):
    _free = "field_grad_free"

    def __init__(self, field, level=2):
        super().__init__()
        self.field = field
        self.ptr = _new("field_grad_create", field.cs.pe.ptr, field.ptr,
                        int(level))

    def compute(self):
        _check(lib().field_grad_compute(self.ptr), "field_grad_compute")

    def set_stencil(self, npoints):
        """7 (default) or 27 points (src/gradient_3d_27pt_fluid.c)."""
        _check(lib().field_grad_stencil_set(self.ptr, int(npoints)),
               "field_grad_stencil_set")

    def get(self):
        nf = self.field.nf
        g = np.zeros((3 * nf,) + self.field.cs.ntotal)
        d = np.zeros((nf,) + self.field.cs.ntotal)
        _check(lib().field_grad_to_host(self.ptr, _dp(g), _dp(d)),
               "field_grad_to_host")
        return g, d


class Hydro(_Obj):
    _free = "hydro_free"

    def __init__(self, cs, precision=FP64):
        super().__init__()
        self.cs = cs
        o = lib().hydro_options_default()
        self.ptr = _new("ludwig_gb_hydro_create", cs.pe.ptr, cs.ptr, None,
                        ctypes.byref(o), int(precision))

    def get(self):
        n = self.cs.ntotal
        rho, u, force = (np.zeros((1,) + n), np.zeros((3,) + n),
                         np.zeros((3,) + n))
        _check(lib().hydro_to_host(self.ptr, _dp(rho), _dp(u), _dp(force)),
               "hydro_to_host")
        return rho, u, force

    def set(self, rho=None, u=None, force=None):
        args = []
        for a in (rho, u, force):
            if a is None:
                args.append(None)
            else:
                a = np.ascontiguousarray(a, dtype=np.float64)
                args.append(a)
        _check(lib().hydro_from_host(self.ptr, *[None if a is None else _dp(a)
                                                 for a in args]),
               "hydro_from_host")

    def f_zero(self):
        _check(lib().hydro_f_zero(self.ptr, _D3(0.0, 0.0, 0.0)),
               "hydro_f_zero")

    def u_zero(self):
        _check(lib().hydro_u_zero(self.ptr, _D3(0.0, 0.0, 0.0)),
               "hydro_u_zero")

    def u_halo(self):
        _check(lib().hydro_u_halo(self.ptr), "hydro_u_halo")

    def io_format(self, fmt_in="binary", fmt_out="binary"):
        _check(lib().hydro_io_record_format_set(self.ptr, _IORF[fmt_in],
                                                _IORF[fmt_out]), "io format")

    def io_write(self, step):
        """hydro_io_write: the fields "rho" and "vel" in the reference's
        format, in the current directory."""
        _check(lib().hydro_io_write(self.ptr, int(step), None),
               "hydro_io_write")

    def io_read(self, step):
        _check(lib().hydro_io_read(self.ptr, int(step), None), "hydro_io_read")

    def velocity_minmax(self, map=None):
        """(umin[3], umax[3], volume flux[3]) over the fluid sites, as
        stats_velocity_minmax prints them."""
        out = np.zeros(9)
        _check(lib().ludwig_gb_stats_velocity_minmax(
            self.ptr, map.ptr if map else None, _dp(out)),
            "stats_velocity_minmax")
        return out[0:3], out[3:6], out[6:9]


class Map(_Obj):
    def __init__(self, cs):
        super().__init__()
        self.cs = cs
        self.options = lib().map_options_default()
        self.ptr = _new("map_create", cs.pe.ptr, cs.ptr,
                        ctypes.byref(self.options))

    def close(self):
        if self.ptr is not None:
            p = ctypes.c_void_p(self.ptr.value)
            lib().map_free(ctypes.byref(p))
            self.ptr = None

    def set_status(self, status):
        s = np.ascontiguousarray(status, dtype=np.uint8)
        assert s.size == self.cs.nsites
        _check(lib().map_status_from_host(
            self.ptr, s.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))),
            "map_status_from_host")


class FeSymm(_Obj):
    _free = "fe_symm_free"

    def __init__(self, cs, phi, dphi, a=-0.0625, b=0.0625, kappa=0.04):
        super().__init__()
        self.ptr = _new("fe_symm_create", cs.pe.ptr, cs.ptr, phi.ptr,
                        dphi.ptr)
        _check(lib().fe_symm_param_set(self.ptr, FeSymmParam(a, b, kappa,
                                                             0.0, 0.0)),
               "fe_symm_param_set")

    def fed_total(self):
        out = ctypes.c_double()
        _check(lib().stats_free_energy_symm(self.ptr, ctypes.byref(out)),
               "stats_free_energy_symm")
        return out.value


class Pth(_Obj):
    _free = "pth_free"

    def __init__(self, cs, method=1):
        super().__init__()
        self.cs = cs
        self.ptr = _new("pth_create", cs.pe.ptr, cs.ptr, int(method))

    def stress_compute(self, fe):
        _check(lib().pth_stress_compute(self.ptr, fe.ptr),
               "pth_stress_compute")

    def get(self):
        s = np.zeros((9,) + self.cs.ntotal)
        _check(lib().pth_to_host(self.ptr, _dp(s)), "pth_to_host")
        return s


class PhiCH(_Obj):
    _free = "phi_ch_free"

    def __init__(self, cs):
        super().__init__()
        info = PhiChInfo(0, 0)
        self.ptr = _new("phi_ch_create", cs.pe.ptr, cs.ptr, None,
                        ctypes.byref(info))


# ---------------------------------------------------------------------------
# The reference's main loop (src/ludwig.c:528-860) for the binary fluid
# ---------------------------------------------------------------------------

def phi_force_calculation(pe, cs, pth, fe, map_, phi, hydro):
    _check(lib().phi_force_calculation(pe.ptr, cs.ptr, None, None, pth.ptr,
                                       fe.ptr, map_.ptr if map_ else None,
                                       phi.ptr, hydro.ptr),
           "phi_force_calculation")


def phi_cahn_hilliard(pch, fe, phi, hydro, map_=None):
    _check(lib().phi_cahn_hilliard(pch.ptr, fe.ptr, phi.ptr,
                                   hydro.ptr if hydro else None,
                                   map_.ptr if map_ else None, None),
           "phi_cahn_hilliard")


class BinaryFluid:
    """All objects of a symmetric binary fluid (D3Q19 M10, 7- or 27-point
    gradients, stress divergence, finite-difference Cahn-Hilliard)."""

    def __init__(self, ntotal, precision=FP64, a=-0.0625, b=0.0625,
                 kappa=0.04, mobility=0.3, eta=0.1, eta_bulk=None, rho0=1.0,
                 fbody=(0.0, 0.0, 0.0), device=0, fp16_scale=0.0,
                 nrelax=0):
        self.pe = PE(device)
        self.cs = Coords(self.pe, ntotal)
        self.phys = Physics(self.pe, rho0=rho0, eta=eta, eta_bulk=eta_bulk,
                            mobility=mobility, fbody=fbody)
        self.lb = LB(self.cs, precision, nrelax=nrelax,
                     fp16_scale=fp16_scale)
        self.phi = Field(self.cs, 1, 2, precision, "phi")
        self.dphi = FieldGrad(self.phi, 2)
        self.hydro = Hydro(self.cs, precision)
        self.map = Map(self.cs)
        self.fe = FeSymm(self.cs, self.phi, self.dphi, a, b, kappa)
        self.pth = Pth(self.cs)
        self.pch = PhiCH(self.cs)
        self.lb.init_rest(rho0)

    def step_reference_order(self, nsteps=1):
        """One call per reference function, in the main-loop order."""
        self.use_physics()
        for _ in range(nsteps):
            self.hydro.f_zero()
            self.phi.halo()
            self.dphi.compute()
            phi_force_calculation(self.pe, self.cs, self.pth, self.fe,
                                  self.map, self.phi, self.hydro)
            self.hydro.u_halo()
            phi_cahn_hilliard(self.pch, self.fe, self.phi, self.hydro,
                              self.map)
            self.hydro.u_zero()
            self.lb.collide(self.hydro, self.map, self.fe)
            self.lb.halo()
            self.lb.propagation()

    def use_physics(self):
        """Make this system's physics the one the step functions read."""
        _check(lib().ludwig_gb_physics_use(self.phys.ptr), "physics_use")

    def step(self, nsteps=1):
        """The fused GB300 step (one kernel per step, graph replay)."""
        self.use_physics()
        _check(lib().ludwig_gb_binary_step(self.lb.ptr, self.phi.ptr,
                                           self.hydro.ptr, self.map.ptr,
                                           self.fe.ptr, int(nsteps)),
               "ludwig_gb_binary_step")

    def step_async(self, nsteps=1):
        self.use_physics()
        _check(lib().ludwig_gb_binary_step_async(self.lb.ptr, self.phi.ptr,
                                                 self.hydro.ptr, self.map.ptr,
                                                 self.fe.ptr, int(nsteps)),
               "ludwig_gb_binary_step_async")

    def state(self):
        rho, u, force = self.hydro.get()
        return {"f": self.lb.get(), "phi": self.phi.get(), "u": u,
                "rho": rho, "force": force}


class BinaryFluidLB:
    """The two-distribution binary fluid (symmetric_lb, ndist = 2): the
    order parameter is the zeroth moment of a second distribution g and
    evolves in the collision (src/collision.c:604-1013).  FP64."""

    def __init__(self, ntotal, a=-0.0625, b=0.0625, kappa=0.04,
                 mobility=0.45, eta=0.1, eta_bulk=None, rho0=1.0,
                 fbody=(0.0, 0.0, 0.0), device=0):
        self.pe = PE(device)
        self.cs = Coords(self.pe, ntotal)
        self.phys = Physics(self.pe, rho0=rho0, eta=eta, eta_bulk=eta_bulk,
                            mobility=mobility, fbody=fbody)
        self.lb = LB(self.cs, FP64, ndist=2)
        self.phi = Field(self.cs, 1, 2, FP64, "phi")
        self.dphi = FieldGrad(self.phi, 2)
        self.hydro = Hydro(self.cs, FP64)
        self.map = Map(self.cs)
        self.fe = FeSymm(self.cs, self.phi, self.dphi, a, b, kappa)
        self.lb.init_rest(rho0)

    def use_physics(self):
        _check(lib().ludwig_gb_physics_use(self.phys.ptr), "physics_use")

    def init_spinodal(self, seed, phi0=0.0, amp=0.02):
        """Spinodal phi moved into g (src/phi_lb_coupler.c:107)."""
        self.phi.init_spinodal(seed, phi0, amp)
        _check(lib().phi_lb_from_field(self.phi.ptr, self.lb.ptr),
               "phi_lb_from_field")

    def step_reference_order(self, nsteps=1):
        """One call per reference function, in the main-loop order."""
        self.use_physics()
        for _ in range(nsteps):
            self.hydro.f_zero()
            _check(lib().phi_lb_to_field(self.phi.ptr, self.lb.ptr),
                   "phi_lb_to_field")
            self.phi.halo()
            self.dphi.compute()
            self.hydro.u_zero()
            self.lb.collide(self.hydro, self.map, self.fe)
            self.lb.halo()
            self.lb.propagation()

    def step(self, nsteps=1):
        """Three kernels per step, streaming folded into the next pull."""
        self.use_physics()
        _check(lib().ludwig_gb_lb2_step(self.lb.ptr, self.phi.ptr,
                                        self.hydro.ptr, self.fe.ptr,
                                        int(nsteps)), "ludwig_gb_lb2_step")

    def state(self):
        _, u, _ = self.hydro.get()
        return {"f": self.lb.get(), "g": self.lb.get_g(),
                "phi": self.phi.get(), "u": u}


def sync():
    _check(lib().ludwig_gb_sync(), "ludwig_gb_sync")


def advection_order(n):
    """Order of the advective fluxes (1, 2, 3) of the per-function
    Cahn-Hilliard and Beris-Edwards steps (src/advection.c:82)."""
    _check(lib().advection_order_set(int(n)), "advection_order_set")


def tune(xchunk, tile_y, min_blocks=0):
    _check(lib().ludwig_gb_tune_set(int(xchunk), int(tile_y),
                                    int(min_blocks)), "tune")


def tune_sites(sites_per_thread):
    """Sites per thread of the float fused step: 2 (packed FP32x2), 1, or
    0 (the default: 2 for FP16 storage, 1 for FP32)."""
    _check(lib().ludwig_gb_tune_sites(int(sites_per_thread)), "tune_sites")


class PinnedState:
    """Page-locked host buffers for the raw state of a BinaryFluid."""

    def __init__(self, system):
        L = lib()
        fb, pb, ub = (ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t())
        _check(L.ludwig_gb_state_bytes(system.lb.ptr, ctypes.byref(fb),
                                       ctypes.byref(pb), ctypes.byref(ub)),
               "state_bytes")
        self.sizes = (fb.value, pb.value, ub.value, pb.value)
        self.bufs = [_new("ludwig_gb_host_alloc", ctypes.c_size_t(b))
                     for b in self.sizes]
        self.bytes_in = fb.value + pb.value + ub.value
        self.bytes_out = fb.value + pb.value + ub.value + pb.value

    def close(self):
        for b in self.bufs:
            lib().ludwig_gb_host_free(b)
        self.bufs = []

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def time_binary(system, nsteps):
    ms = ctypes.c_double()
    s = system
    _check(lib().ludwig_gb_time_binary(s.lb.ptr, s.phi.ptr, s.hydro.ptr,
                                       s.map.ptr, s.fe.ptr, int(nsteps),
                                       ctypes.byref(ms)), "time_binary")
    return ms.value


def time_binary_e2e_overlap(system, pin_in, pin_out, nsteps):
    """End-to-end time (ms) of nsteps steps, each uploading the same host
    input (pin_in, filled here from the system's state) and downloading
    its result to pin_out, with the copies of consecutive steps
    overlapped."""
    ms = ctypes.c_double()
    s = system
    L = lib()
    _check(L.ludwig_gb_state_to_host_async(s.lb.ptr, s.phi.ptr, s.hydro.ptr,
                                           *pin_in.bufs[:3]), "state_to_host")
    sync()
    _check(L.ludwig_gb_time_binary_e2e_overlap(
        s.lb.ptr, s.phi.ptr, s.hydro.ptr, s.map.ptr, s.fe.ptr, int(nsteps),
        *pin_in.bufs[:3], *pin_out.bufs, ctypes.byref(ms)),
        "time_binary_e2e_overlap")
    return ms.value


def time_binary_e2e(system, pinned, nsteps):
    ms = ctypes.c_double()
    s = system
    L = lib()
    _check(L.ludwig_gb_state_to_host_async(s.lb.ptr, s.phi.ptr, s.hydro.ptr,
                                           *pinned.bufs[:3]), "state_to_host")
    sync()
    _check(L.ludwig_gb_time_binary_e2e(s.lb.ptr, s.phi.ptr, s.hydro.ptr,
                                       s.map.ptr, s.fe.ptr, int(nsteps),
                                       *pinned.bufs, ctypes.byref(ms)),
           "time_binary_e2e")
    return ms.value


# ---------------------------------------------------------------------------
# Cholesteric liquid crystal
# ---------------------------------------------------------------------------

class FeLC(_Obj):
    """fe_lc_t: Landau-de Gennes free energy (src/blue_phase.c)."""
    _free = "fe_lc_free"

    def __init__(self, cs, q, dq, a0=0.01, gamma=3.0, kappa0=0.01,
                 kappa1=0.01, pitch=32.0, xi=0.7, redshift=1.0,
                 amplitude=-0.2, q0=None, epsilon=0.0, e0=(0.0, 0.0, 0.0)):
        super().__init__()
        self.ptr = _new("fe_lc_create", cs.pe.ptr, cs.ptr, None, q.ptr,
                        dq.ptr)
        p = FeLcParam()
        p.a0, p.gamma, p.kappa0, p.kappa1 = a0, gamma, kappa0, kappa1
        p.q0 = (2.0 * 3.1415926535897932385 / pitch) if q0 is None else q0
        p.xi, p.redshift, p.amplitude0, p.coswt = xi, redshift, amplitude, 1.0
        # dielectric anisotropy (fe_lc_param_set divides it by 12 pi) and
        # a static external field
        p.epsilon = epsilon
        for a in range(3):
            p.e0[a] = e0[a]
        self.param = p
        self.dq = dq
        _check(lib().fe_lc_param_set(self.ptr, ctypes.byref(p)),
               "fe_lc_param_set")

    def fed_total(self, recompute=True):
        """Total free energy (FP64 fields).  recompute: take the gradients
        of the current q first; otherwise use the stored ones (those of
        the last step, as the reference's statistics do after a step)."""
        if recompute:
            self.dq.compute()
        out = ctypes.c_double()
        _check(lib().stats_free_energy_lc(self.ptr, ctypes.byref(out)),
               "stats_free_energy_lc")
        return out.value

    def stats_info(self, map=None, recompute=True):
        """The columns of the reference's "[fe]" line: (f, v, f/v,
        f_bulk/v, f_grad/v, redshift) over the fluid sites."""
        if recompute:
            self.dq.compute()
        out = np.zeros(6)
        _check(lib().ludwig_gb_fe_lc_stats_info(
            self.ptr, map.ptr if map else None, _dp(out)), "fe_lc_stats_info")
        return out


class BerisEdw(_Obj):
    _free = "beris_edw_free"

    def __init__(self, cs, xi=0.7, gamma=0.5):
        super().__init__()
        self.cs = cs
        self.ptr = _new("beris_edw_create", cs.pe.ptr, cs.ptr, None)
        p = BerisEdwParam(xi, gamma, 0, 0.0)
        _check(lib().beris_edw_param_set(self.ptr, ctypes.byref(p)),
               "beris_edw_param_set")

    def update(self, fe, q, dq, hydro, map_=None):
        _check(lib().beris_edw_update(self.ptr, fe.ptr, q.ptr, dq.ptr,
                                      hydro.ptr if hydro else None, None,
                                      map_.ptr if map_ else None, None),
               "beris_edw_update")

    def h(self):
        a = np.zeros((5,) + self.cs.ntotal)
        _check(lib().beris_edw_h_to_host(self.ptr, _dp(a)), "be_h")
        return a


class LiquidCrystal:
    """All objects of the cholesteric liquid crystal (Landau-de Gennes,
    Beris-Edwards), with or without hydrodynamics."""

    def __init__(self, ntotal, eta=0.5, gamma_rot=0.5, device=0,
                 precision=FP64, eta_bulk=None, hydrodynamics=True, **lc):
        self.pe = PE(device)
        self.cs = Coords(self.pe, ntotal)
        self.phys = Physics(self.pe, rho0=1.0, eta=eta, eta_bulk=eta_bulk)
        # hydrodynamics off: Q relaxes without flow (no force, no LB step),
        # as the reference's "hydrodynamics off"
        self.hydrodynamics = bool(hydrodynamics)
        self.lb = LB(self.cs, precision)
        self.q = Field(self.cs, 5, 2, precision, "q")
        self.dq = FieldGrad(self.q, 2)
        self.hydro = Hydro(self.cs, precision)
        self.map = Map(self.cs)
        self.fe = FeLC(self.cs, self.q, self.dq, **lc)
        self.be = BerisEdw(self.cs, xi=self.fe.param.xi, gamma=gamma_rot)
        self.pth = Pth(self.cs)
        self.lb.init_rest(1.0)

    def init_o8m(self, euler_angles=(0.0, 0.0, 0.0)):
        """Blue phase I; euler_angles (degrees, Z-X-Z) rotate it."""
        _check(lib().blue_phase_O8M_init(self.cs.ptr,
                                         ctypes.byref(self.fe.param),
                                         self.q.ptr, _D3(*euler_angles)),
               "o8m")

    def init_o2(self, euler_angles=(0.0, 0.0, 0.0)):
        """Blue phase II; euler_angles (degrees, Z-X-Z) rotate it."""
        _check(lib().blue_phase_O2_init(self.cs.ptr,
                                        ctypes.byref(self.fe.param),
                                        self.q.ptr, _D3(*euler_angles)),
               "o2")

    def init_random(self):
        """Random uniaxial directors (the reference's seed 13)."""
        _check(lib().blue_phase_random_q_init(self.cs.ptr,
                                              ctypes.byref(self.fe.param),
                                              self.q.ptr), "random_q")

    def init_cholesteric(self, axis):
        """Cholesteric helix along axis 0, 1 or 2 (X, Y, Z)."""
        _check(lib().blue_phase_twist_init(self.cs.ptr,
                                           ctypes.byref(self.fe.param),
                                           self.q.ptr, int(axis)), "twist")

    def random_rectangle(self, rmin, rmax):
        """Random directors (amplitude 0.01) in the box rmin..rmax
        (1-based, inclusive) on top of the current Q."""
        a = (ctypes.c_int * 3)(*rmin)
        b = (ctypes.c_int * 3)(*rmax)
        _check(lib().blue_phase_random_q_rectangle(
            self.cs.ptr, ctypes.byref(self.fe.param), self.q.ptr, a, b),
            "random_q_rectangle")

    def init_nematic(self, n):
        _check(lib().blue_phase_nematic_init(self.cs.ptr,
                                             ctypes.byref(self.fe.param),
                                             self.q.ptr, _D3(*n)), "nematic")

    def step_reference_order(self, nsteps=1):
        for _ in range(nsteps):
            if not self.hydrodynamics:
                self.q.halo()
                self.dq.compute()
                self.be.update(self.fe, self.q, self.dq, None, self.map)
                continue
            self.hydro.f_zero()
            self.q.halo()
            self.dq.compute()
            phi_force_calculation(self.pe, self.cs, self.pth, self.fe,
                                  self.map, self.q, self.hydro)
            self.hydro.u_halo()
            self.be.update(self.fe, self.q, self.dq, self.hydro, self.map)
            self.hydro.u_zero()
            self.lb.collide(self.hydro, self.map, self.fe)
            self.lb.halo()
            self.lb.propagation()

    def step(self, nsteps=1):
        """The fused GB300 LC step (two kernels per step)."""
        _check(lib().ludwig_gb_lc_step(self.lb.ptr, self.q.ptr,
                                       self.hydro.ptr, self.map.ptr,
                                       self.fe.ptr, self.be.ptr,
                                       int(nsteps)), "ludwig_gb_lc_step")

    def time(self, nsteps):
        """Device time (ms) of nsteps fused LC steps."""
        ms = ctypes.c_double()
        _check(lib().ludwig_gb_time_lc(self.lb.ptr, self.q.ptr,
                                       self.hydro.ptr, self.map.ptr,
                                       self.fe.ptr, self.be.ptr, int(nsteps),
                                       ctypes.byref(ms)), "ludwig_gb_time_lc")
        return ms.value

    def state(self):
        rho, u, force = self.hydro.get()
        return {"f": self.lb.get(), "q": self.q.get(), "u": u, "rho": rho,
                "force": force}


# ---------------------------------------------------------------------------
# Ensembles of independent boxes
# ---------------------------------------------------------------------------

def box_param(ntotal, eta=0.1, a=-0.0625, b=0.0625, kappa=0.04,
              mobility=0.3, seed=8361235, rho0=1.0, phi0=0.0, noise=0.02):
    p = BoxParam()
    for i in range(3):
        p.ntotal[i] = int(ntotal[i])
    p.rho0, p.eta, p.eta_bulk = rho0, eta, 0.0
    p.a, p.b, p.kappa, p.mobility = a, b, kappa, mobility
    p.seed, p.phi0, p.noise = int(seed), phi0, noise
    return p


class Ensemble:
    """ludwig_gb_ensemble_t: boxes advanced together, one launch a step."""

    def __init__(self, params, precision=FP32, device=0):
        self.pe = PE(device)
        self.params = list(params)
        arr = (BoxParam * len(self.params))(*self.params)
        self.ptr = _new("ludwig_gb_ensemble_create", len(self.params), arr,
                        int(precision))

    def close(self):
        if self.ptr is not None:
            lib().ludwig_gb_ensemble_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def step(self, n=1):
        _check(lib().ludwig_gb_ensemble_step(self.ptr, int(n)), "ens_step")

    def time(self, n):
        ms = ctypes.c_double()
        _check(lib().ludwig_gb_ensemble_time(self.ptr, int(n),
                                             ctypes.byref(ms)), "ens_time")
        return ms.value

    def tune(self, xchunk, tile_y, min_blocks=0):
        _check(lib().ludwig_gb_ensemble_tune_set(self.ptr, int(xchunk),
                                                 int(tile_y),
                                                 int(min_blocks)), "tune")

    def autotune(self, trial_steps=10):
        best = (ctypes.c_int * 3)()
        ms = ctypes.c_double()
        _check(lib().ludwig_gb_ensemble_autotune(self.ptr, int(trial_steps),
                                                 best, ctypes.byref(ms)),
               "autotune")
        return tuple(best), ms.value

    def box(self, b, f=False):
        L = tuple(self.params[b].ntotal)
        phi, u, rho = (np.zeros((1,) + L), np.zeros((3,) + L),
                       np.zeros((1,) + L))
        ff = np.zeros((NVEL,) + L) if f else None
        _check(lib().ludwig_gb_ensemble_box_get(
            self.ptr, int(b), _dp(ff) if f else None, _dp(phi), _dp(u),
            _dp(rho)), "box_get")
        out = {"phi": phi, "u": u, "rho": rho}
        if f:
            out["f"] = ff
        return out

    def set_phi(self, b, phi):
        a = np.ascontiguousarray(phi, dtype=np.float64)
        _check(lib().ludwig_gb_ensemble_box_set_phi(self.ptr, int(b), _dp(a)),
               "set_phi")

    def check(self):
        n = ctypes.c_int()
        _check(lib().ludwig_gb_ensemble_check(self.ptr, ctypes.byref(n)),
               "check")
        return n.value

    def active(self, b):
        a = ctypes.c_int()
        _check(lib().ludwig_gb_ensemble_box_active(self.ptr, int(b),
                                                   ctypes.byref(a)), "active")
        return bool(a.value)

    def sites(self):
        n = ctypes.c_longlong()
        _check(lib().ludwig_gb_ensemble_sites(self.ptr, ctypes.byref(n)),
               "sites")
        return n.value


def ensemble_uneven_boxes(nbox=64, seed=20261203, edges=(32, 48, 64, 96)):
    """64 uneven boxes: edges drawn per axis from `edges`, viscosity
    U[0.02, 0.2], kappa U[0.02, 0.08], A = -B with |A| U[0.03, 0.1],
    mobility min(0.45, 1/(12 (12 kappa + 2|A|))) (half the stability
    bound of the explicit 7-point Cahn-Hilliard step in the saturated
    phases, where the bulk free energy's curvature is 2|A|), phi0 +-0.01
    from per-box seeds."""
    rng = np.random.default_rng(seed)
    out = []
    for k in range(nbox):
        n = [int(rng.choice(edges)) for _ in range(3)]
        eta = float(rng.uniform(0.02, 0.2))
        kappa = float(rng.uniform(0.02, 0.08))
        amag = float(rng.uniform(0.03, 0.1))
        mob = min(0.45, 1.0 / (12.0 * (12.0 * kappa + 2.0 * amag)))
        out.append(box_param(n, eta=eta, a=-amag, b=amag, kappa=kappa,
                             mobility=mob, seed=1000 + 17 * k))
    return out


# ---------------------------------------------------------------------------
# Learned corrector (no counterpart in the reference)
# ---------------------------------------------------------------------------

def _fp(a):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(_F)


def _f3(v, n):
    a = np.ascontiguousarray(np.asarray(v, dtype=np.float32).reshape(n))
    return a


class Corrector(_Obj):
    """The 3x3x3 convolutional corrector of a 2x-coarsened binary fluid.

    Device arrays are passed as integer device pointers (for example
    ``tensor.data_ptr()`` of a contiguous float32 CUDA tensor).
    """
    _free = "ludwig_gb_cnn_free"

    def __init__(self, ncoarse, seed=1):
        super().__init__()
        self.n = tuple(int(v) for v in ncoarse)
        self.ptr = _new("ludwig_gb_cnn_create", _I3(*self.n),
                        ctypes.c_ulonglong(seed))

    @staticmethod
    def nparams():
        return int(lib().ludwig_gb_cnn_nparams())

    @property
    def nsites(self):
        return self.n[0] * self.n[1] * self.n[2]

    def params(self):
        h = np.zeros(self.nparams(), dtype=np.float32)
        _check(lib().ludwig_gb_cnn_params_get(self.ptr, _fp(h)), "params_get")
        return h

    def set_params(self, p):
        h = np.ascontiguousarray(p, dtype=np.float32)
        assert h.size == self.nparams()
        _check(lib().ludwig_gb_cnn_params_set(self.ptr, _fp(h)), "params_set")

    def grads(self):
        h = np.zeros(self.nparams(), dtype=np.float32)
        _check(lib().ludwig_gb_cnn_grads_get(self.ptr, _fp(h)), "grads_get")
        return h

    def set_scales(self, in_off, in_scale, out_scale):
        a, b, c = _f3(in_off, 5), _f3(in_scale, 5), _f3(out_scale, 4)
        _check(lib().ludwig_gb_cnn_scales_set(self.ptr, _fp(a), _fp(b),
                                              _fp(c)), "scales_set")

    def scales(self):
        a = np.zeros(5, np.float32)
        b = np.zeros(5, np.float32)
        c = np.zeros(4, np.float32)
        _check(lib().ludwig_gb_cnn_scales_get(self.ptr, _fp(a), _fp(b),
                                              _fp(c)), "scales_get")
        return a, b, c

    def forward(self, in5, out4):
        _check(lib().ludwig_gb_cnn_forward(self.ptr, in5, out4), "forward")

    def forward_n(self, in5s, out4s):
        """Several forward passes back to back (device pointers), one error
        check after the last."""
        n = len(in5s)
        a = (ctypes.c_void_p * max(n, 1))(*in5s)
        b = (ctypes.c_void_p * max(n, 1))(*out4s)
        _check(lib().ludwig_gb_cnn_forward_n(self.ptr, n, a, b), "forward_n")

    def train_steps(self, in5s, t4s, lr):
        """Several Adam steps back to back without reading the losses."""
        n = len(in5s)
        a = (ctypes.c_void_p * max(n, 1))(*in5s)
        b = (ctypes.c_void_p * max(n, 1))(*t4s)
        _check(lib().ludwig_gb_cnn_train_steps(self.ptr, n, a, b, float(lr),
                                               None), "train_steps")

    def loss_grad(self, in5, t4):
        loss = ctypes.c_double()
        _check(lib().ludwig_gb_cnn_loss_grad(self.ptr, in5, t4,
                                             ctypes.byref(loss)), "loss_grad")
        return loss.value

    def train_step(self, in5, t4, lr):
        loss = ctypes.c_double()
        _check(lib().ludwig_gb_cnn_train_step(self.ptr, in5, t4, float(lr),
                                              ctypes.byref(loss)),
               "train_step")
        return loss.value

    def correct(self, system):
        _check(lib().ludwig_gb_cnn_correct(self.ptr, system.lb.ptr,
                                           system.phi.ptr, system.hydro.ptr),
               "cnn_correct")

    def line_reuse(self, mode=1):
        """Line-reuse convolutions where nz is a multiple of 128: 1 (planes
        of 8 channels), 2 (swizzled rows), 3 (planes, the three z taps of
        a line in one MMA; nz = 128 only, 1 otherwise), 4 (as 3, and the
        last layer with its y taps folded into the MMAs as well; nz = 128
        only), 5 (as 4 on swizzled lines; nz = 128 only), 0/False (one box
        per tap).  The default is 5 where nz = 128, else 1."""
        _check(lib().ludwig_gb_cnn_line_reuse(self.ptr, int(mode)),
               "cnn_line_reuse")

    def conv3(self, a, w, b, flip, out):
        _check(lib().ludwig_gb_cnn_conv3(self.ptr, a, w, b, int(flip), out),
               "cnn_conv3")

    def wgrad3(self, g, a, dw):
        _check(lib().ludwig_gb_cnn_wgrad3(self.ptr, g, a, dw), "cnn_wgrad3")


def coarse_restrict(fine, coarse):
    """Coarse FP32 state from a fine FP32 state of twice the extents."""
    _check(lib().ludwig_gb_coarse_restrict(fine.lb.ptr, fine.phi.ptr,
                                           fine.hydro.ptr, coarse.lb.ptr,
                                           coarse.phi.ptr, coarse.hydro.ptr),
           "coarse_restrict")


def fields_restrict(fine, out5, ncoarse):
    _check(lib().ludwig_gb_fields_restrict(fine.phi.ptr, fine.hydro.ptr,
                                           fine.lb.ptr, out5,
                                           _I3(*ncoarse)), "fields_restrict")


def fields_pack(system, out5):
    _check(lib().ludwig_gb_fields_pack(system.phi.ptr, system.hydro.ptr,
                                       system.lb.ptr, out5), "fields_pack")

"""ctypes mirror of include/song2.h.

This module is the binding a maintainer of the reference would add to drive
the C ABI from Python (the reference itself is driven from C, through the same
entry points).  Every structure here matches song2.h field by field.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libsong2.so")

SONG2_ERRLEN = 1024
SONG2_MAX_M = 5
SONG2_MAX_L = 64

# status codes
SONG2_OK, SONG2_E_MAXSTEPS, SONG2_E_HMIN, SONG2_E_NAN, SONG2_E_NEWTON, SONG2_E_SINGULAR, SONG2_E_CONFIG = range(7)
# initial conditions
SONG2_IC_AD, SONG2_IC_AD_FIRST_ORDER, SONG2_IC_ZERO = range(3)
# precision
SONG2_PREC_FP64, SONG2_PREC_MIXED = 0, 1
# radiation-streaming approximation
SONG2_RSA_NONE, SONG2_RSA_MD, SONG2_RSA_MD_WITH_REIO = 0, 1, 2
# tau_c/tau at which photons free-stream (radiation_streaming_trigger_tau_c_over_tau_song)
RSA_TRIGGER_TAU_C_OVER_TAU = 10.0

# background columns
(BG_LN_A, BG_LN_HC, BG_HC_PRIME_TAU2, BG_LN_RHO_G, BG_LN_RHO_B, BG_LN_RHO_CDM, BG_LN_RHO_UR,
 BG_LN_KAPPA_DOT, BG_KAPPA, BG_SIZE) = range(10)

# first-order quantities
(FO_PHI, FO_PSI, FO_PHI_P, FO_PSI_P, FO_PHI_PP, FO_DELTA_G, FO_V_G, FO_DELTA_B, FO_V_B,
 FO_DELTA_B_P, FO_V_B_P, FO_DELTA_CDM, FO_V_CDM, FO_V_CDM_P, FO_DELTA_UR, FO_V_UR,
 FO_DIPOLE_B, FO_DIPOLE_CDM, FO_I) = range(19)


def fo_size(fo_l_max):
    return FO_I + 4 * (fo_l_max + 1)


class Cosmo(C.Structure):
    _fields_ = [("h", C.c_double), ("omega_b", C.c_double), ("omega_cdm", C.c_double),
                ("N_eff", C.c_double), ("T_cmb", C.c_double), ("YHe", C.c_double), ("z_reio", C.c_double)]


class Spec(C.Structure):
    _fields_ = [
        ("l_max_g", C.c_int), ("l_max_pol_g", C.c_int), ("l_max_ur", C.c_int),
        ("l_max_los_t", C.c_int), ("l_max_los_p", C.c_int),
        ("m_size", C.c_int), ("m", C.c_int * SONG2_MAX_M),
        ("has_polarization2", C.c_int),
        ("has_quadratic_sources", C.c_int), ("has_quadratic_liouville", C.c_int),
        ("has_quadratic_collision", C.c_int),
        ("tight_coupling", C.c_int),
        ("tca_trigger_tau_c_over_tau_h", C.c_double), ("tca_trigger_tau_c_over_tau_k", C.c_double),
        ("ic", C.c_int), ("primordial_local_fnl_phi", C.c_double),
        ("has_pure_scattering_in_los", C.c_int), ("has_quad_scattering_in_los", C.c_int),
        ("has_pure_metric_in_los", C.c_int), ("has_quad_metric_in_los", C.c_int),
        ("has_time_delay_in_los", C.c_int), ("has_redshift_in_los", C.c_int),
        ("has_lensing_in_los", C.c_int),
        ("has_sw", C.c_int), ("has_isw", C.c_int), ("use_exponential_potentials", C.c_int),
        ("has_source_T", C.c_int), ("has_source_E", C.c_int), ("has_source_B", C.c_int),
        ("has_source_delta_cdm", C.c_int),
        ("rtol", C.c_double), ("threshold", C.c_double), ("max_steps", C.c_int),
        ("start_small_k_at_tau_c_over_tau_h", C.c_double),
        ("start_large_k_at_tau_h_over_tau_k", C.c_double),
        ("tol_tau_approx", C.c_double),
        ("k_size", C.c_int), ("k", C.POINTER(C.c_double)),
        ("k3_size", C.POINTER(C.c_int)), ("k3", C.POINTER(C.c_double)),
        ("tau_size", C.c_int), ("tau", C.POINTER(C.c_double)),
        ("n_classes", C.c_int), ("class_l_max", C.POINTER(C.c_int)), ("class_m_max", C.POINTER(C.c_int)),
        ("triplet_class", C.POINTER(C.c_int)),
        ("use_delta_tilde_in_los", C.c_int),
        ("l_max_los_quadratic_t", C.c_int), ("l_max_los_quadratic_p", C.c_int),
        ("rescale_cmb_sources", C.c_int),
        ("radiation_streaming_approximation", C.c_int),
        ("radiation_streaming_trigger_tau_over_tau_k", C.c_double),
    ]


class Tables(C.Structure):
    _fields_ = [
        ("tau0", C.c_double), ("a_eq", C.c_double),
        ("bg_size", C.c_int), ("bg_lntau0", C.c_double), ("bg_dlntau", C.c_double),
        ("bg", C.POINTER(C.c_double)), ("bg_dd", C.POINTER(C.c_double)),
        ("fo_k_size", C.c_int), ("fo_tau_size", C.c_int),
        ("fo_lntau0", C.c_double), ("fo_dlntau", C.c_double),
        ("fo_l_max", C.c_int), ("fo_size", C.c_int),
        ("fo", C.POINTER(C.c_double)), ("fo_dd", C.POINTER(C.c_double)),
        ("tau_free_streaming", C.c_double),
    ]


class LosSpec(C.Structure):
    """song2_los_spec: the transfer2/bessel2 parameters of the line-of-sight integration."""
    _fields_ = [
        ("l_size", C.c_int), ("l", C.POINTER(C.c_int)),
        ("k3_sampling", C.c_int), ("q_linstep", C.c_double),
        ("tau_sampling", C.c_int), ("tau_linstep", C.c_double),
        ("k3_interpolation", C.c_int), ("time_interpolation", C.c_int), ("bessel_interpolation", C.c_int),
        ("k3_extrapolation", C.c_int),
        ("extra_k3_oscillations_left", C.c_double), ("extra_k3_oscillations_right", C.c_double),
        ("x_step", C.c_double), ("x_max", C.c_double),
        ("j_cut", C.c_double), ("J_cut", C.c_double), ("bessel_tol_x_min", C.c_double),
        ("tau0", C.c_double), ("tau_rec", C.c_double),
    ]


class BispectraSpec(C.Structure):
    """song2_bispectra_spec: fields, r and q grids, P(q) and the first-order transfers."""
    _fields_ = [
        ("bf_size", C.c_int), ("bf", C.POINTER(C.c_int)),
        ("r_size", C.c_int), ("r", C.POINTER(C.c_double)),
        ("q_size", C.c_int), ("q", C.POINTER(C.c_double)),
        ("pk", C.POINTER(C.c_double)), ("transfer1", C.POINTER(C.c_double)),
        ("k1_interpolation", C.c_int), ("k2_interpolation", C.c_int),
    ]


K3_SAMPLING_CLASS, K3_SAMPLING_BESSEL = 0, 1
TAU_SAMPLING_SOURCES, TAU_SAMPLING_CUSTOM, TAU_SAMPLING_BESSEL = 0, 1, 2
INTERP_LINEAR, INTERP_CUBIC = 0, 1
K3_EXTRAP_NONE, K3_EXTRAP_FLAT = 0, 1


class Params(C.Structure):
    """song2_params: the grid settings of a parameter file."""
    _fields_ = [("k_sampling", C.c_int), ("k_min", C.c_double), ("k_max", C.c_double), ("k_size", C.c_int),
                ("k3_sampling", C.c_int), ("k3_size", C.c_int), ("custom_tau", C.c_int), ("tau_sampling", C.c_int),
                ("tau_ini", C.c_double), ("tau_end", C.c_double), ("tau_size", C.c_int),
                ("l_max_scalars", C.c_int), ("l_logstep", C.c_double), ("l_linstep", C.c_int),
                ("k_min_tau0", C.c_double), ("k_max_tau0_over_l_max", C.c_double), ("k_step_sub", C.c_double),
                ("k_step_super", C.c_double), ("k_logstep_super", C.c_double), ("k_step_transition", C.c_double),
                ("k_per_decade_for_pk", C.c_double), ("k_per_decade_for_bao", C.c_double),
                ("k_bao_center", C.c_double), ("k_bao_width", C.c_double), ("k_max_for_pk", C.c_double),
                ("h", C.c_double), ("k3_size_min", C.c_int), ("has_cmb", C.c_int), ("has_lss", C.c_int),
                ("tau_stepsize", C.c_double), ("tau_late_boost", C.c_double), ("tau_start_c_over_h", C.c_double),
                ("bi_k1_interpolation", C.c_int), ("bi_k2_interpolation", C.c_int), ("bi_r_size", C.c_int)]


SAMPLING_LIN, SAMPLING_LOG, SAMPLING_SMART, SAMPLING_SYM, SAMPLING_THETA12 = 0, 1, 2, 3, 4


class Launch(C.Structure):
    _fields_ = [("warp_team", C.c_int), ("teams_per_cta", C.c_int), ("threads_per_team", C.c_int),
                ("lu_in_smem", C.c_int)]


class TripletStats(C.Structure):
    _fields_ = [("status", C.c_int32), ("n_steps", C.c_int32), ("n_rejected", C.c_int32),
                ("n_rhs", C.c_int32), ("n_jac", C.c_int32), ("n_lu", C.c_int32),
                ("n_newton_fail", C.c_int32), ("sources_calls", C.c_int32), ("retried", C.c_int32)]


STATS_DTYPE = np.dtype([("status", np.int32), ("n_steps", np.int32), ("n_rejected", np.int32),
                        ("n_rhs", np.int32), ("n_jac", np.int32), ("n_lu", np.int32),
                        ("n_newton_fail", np.int32), ("sources_calls", np.int32), ("retried", np.int32)])

# Every extern "C" symbol declared in include/song2.h, with its ctypes signature.
_P = C.c_void_p
_D = C.c_double
_I = C.c_int
_PD = C.POINTER(C.c_double)
_PI = C.POINTER(C.c_int)
SIGNATURES = {
    "song2_fo_size": (_I, [_I]),
    "song2_n_triplets": (C.c_int64, [C.POINTER(Spec)]),
    "song2_tp2_size": (_I, [C.POINTER(Spec)]),
    "song2_pair_offset": (C.c_int64, [C.POINTER(Spec), _I, _I]),
    "song2_sources_per_type": (C.c_int64, [C.POINTER(Spec)]),
    "song2_store_sources": (_I, [C.POINTER(Spec), C.POINTER(C.c_double), C.c_char_p, _I, C.c_char_p]),
    "song2_load_sources": (_I, [C.POINTER(Spec), C.POINTER(C.c_double), C.c_char_p, _I, C.c_char_p]),
    "song2_spec_defaults": (None, [C.POINTER(Spec)]),
    "song2_background_compute": (_I, [C.POINTER(Cosmo), _I, _PD, _PD, _PD, _PD, _PD, _PD, C.c_char_p]),
    "song2_spline_uniform": (None, [_I, _I, _D, _PD, _PD]),
    "song2_first_order_from_provider": (_I, [C.POINTER(Spec), _I, _I, _D, _D, C.c_void_p, C.c_void_p, _I, _PI,
                                             _PD, _PD, C.POINTER(Tables), C.c_char_p]),
    "song2_background_from_provider": (_I, [_I, _D, _D, C.c_void_p, C.c_void_p, _PD, _PD, C.POINTER(Tables),
                                            C.c_char_p]),
    "song2_coupling_c_minus": (_D, [_I, _I, _I]),
    "song2_coupling_c_plus": (_D, [_I, _I, _I]),
    "song2_coupling_d_minus": (_D, [_I, _I, _I]),
    "song2_coupling_d_plus": (_D, [_I, _I, _I]),
    "song2_coupling_d_zero": (_D, [_I, _I, _I]),
    "song2_delta_tilde_coupling": (_D, [_I, _I, _I, _I, _I, _I]),
    "song2_free_streaming_time": (_D, [C.POINTER(Tables), _D]),
    "song2_k_grid": (_I, [_I, _D, _D, _I, _PD]),
    "song2_k3_grids": (_I, [_PD, _I, _I, _I, _PI, _PD, C.c_char_p]),
    "song2_tau_grid": (_I, [_I, _D, _D, _I, _PD]),
    "song2_start_time": (_I, [C.POINTER(Spec), C.POINTER(Tables), _D, _D, _PD, C.c_char_p]),
    "song2_shard_items": (C.c_int64, [C.POINTER(Spec), _I, _I, C.POINTER(C.c_int64)]),
    "song2_ctx_create": (_I, [C.POINTER(Spec), C.POINTER(Tables), _I, C.POINTER(_P), C.c_char_p]),
    "song2_ctx_create_shard": (_I, [C.POINTER(Spec), C.POINTER(Tables), _I, _I, _I, C.POINTER(_P), C.c_char_p]),
    "song2_ctx_create_list": (_I, [C.POINTER(Spec), C.POINTER(Tables), _I, C.POINTER(C.c_int64), C.c_int64,
                                   C.POINTER(_P), C.c_char_p]),
    "song2_ctx_create_ex": (_I, [C.POINTER(Spec), C.POINTER(Tables), _I, C.c_void_p, _I, _I, C.POINTER(_P),
                                 C.c_char_p]),
    "song2_ctx_get_launch": (None, [_P, C.c_void_p, C.POINTER(_I), C.POINTER(_I), C.POINTER(C.c_size_t)]),
    "song2_autotune": (_I, [C.POINTER(Spec), C.POINTER(Tables), _I, _I, C.c_void_p, _PD, C.c_char_p]),
    "song2_ctx_destroy": (_I, [_P]),
    "song2_ctx_run": (_I, [_P, _P, C.c_char_p]),
    "song2_ctx_run_graph": (_I, [_P, _P, C.c_char_p]),
    "song2_ctx_run_part": (_I, [_P, _I, _I, _P, C.c_char_p]),
    "song2_ctx_enqueue_part": (_I, [_P, _I, _I, _P, C.c_char_p]),
    "song2_ctx_device_sources": (_P, [_P]),
    "song2_ctx_device_stats": (_P, [_P]),
    "song2_ctx_download": (_I, [_P, _PD, C.POINTER(TripletStats), C.c_char_p]),
    "song2_ctx_last_kernel_ms": (_D, [_P]),
    "song2_ctx_last_launches": (_I, [_P]),
    "song2_ctx_phase_cycles": (_I, [_P, C.POINTER(C.c_uint64), _I]),
    "song2_gpu_evolve": (_I, [C.POINTER(Spec), C.POINTER(Tables), _I, _P, C.POINTER(TripletStats),
                              C.c_char_p]),
    "song2_gpu_evolve_noalloc": (_I, [C.POINTER(Spec), C.POINTER(Tables), _I, C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.c_char_p]),
    "song2_gpu_first_order": (_I, [C.POINTER(Spec), C.POINTER(Tables), _I, _I, _D, _D, _PD, C.c_char_p]),
    "song2_los_defaults": (None, [C.POINTER(LosSpec), C.POINTER(Spec), C.POINTER(Tables)]),
    "song2_params_defaults": (None, [C.POINTER(Params)]),
    "song2_write_sources_k": (_I, [C.POINTER(Spec), C.POINTER(Tables), _PD, _I, _I, C.c_char_p, C.c_char_p]),
    "song2_write_sources_tau": (_I, [C.POINTER(Spec), C.POINTER(Tables), _PD, _I, C.c_char_p, C.c_char_p]),
    "song2_sound_horizon": (_D, [C.POINTER(Tables), _D]),
    "song2_tau_grid_class": (_I, [C.POINTER(Tables), _D, _D, _D, _D, _I, _PD, C.c_char_p]),
    "song2_k3_grids_theta12": (_I, [_PD, _I, _I, _PI, _PD, C.c_char_p]),
    "song2_read_cosmo": (_I, [C.c_char_p, C.c_char_p, C.POINTER(Cosmo), C.c_char_p]),
    "song2_k_grid_smart": (_I, [C.POINTER(Params), _D, _D, _I, _PD, C.c_char_p]),
    "song2_k3_grids_smart": (_I, [_PD, _I, _I, _PI, _PD, C.c_char_p]),
    "song2_read_params": (_I, [C.c_char_p, C.c_char_p, C.POINTER(Spec), C.POINTER(Params), C.POINTER(LosSpec),
                               C.c_char_p]),
    "song2_l_list": (_I, [_I, _D, _I, _PI]),
    "song2_recombination_time": (_D, [C.POINTER(Tables)]),
    "song2_transfer_types": (_I, [C.POINTER(Spec), C.POINTER(LosSpec), _PI, _PI, _PI]),
    "song2_transfer_k_grids": (C.c_int64, [C.POINTER(Spec), C.POINTER(LosSpec), _PI, _PI, _PI, _PD, C.c_char_p]),
    "song2_wigner3j_row": (_I, [_I, _I, _I, _I, _PI, _PI, _PD, _I]),
    "song2_los_create": (_I, [C.POINTER(Spec), C.POINTER(LosSpec), C.POINTER(_P), C.c_char_p]),
    "song2_los_destroy": (None, [_P]),
    "song2_los_transfer_size": (C.c_int64, [_P]),
    "song2_los_run": (_I, [_P, _P, _P, _P, C.c_char_p]),
    "song2_los_last_ms": (C.c_float, [_P]),
    "song2_los_tables_ms": (C.c_float, [_P]),
    "song2_los_table_sizes": (None, [_P, _PI, _PI, _PI, _PI, _PI]),
    "song2_los_tables": (_I, [_P, _PI, _PD, _PD, _PI, C.c_char_p]),
    "song2_gpu_transfer": (_I, [C.POINTER(Spec), C.POINTER(LosSpec), _PD, _PD, C.c_char_p]),
    "song2_bispectra_configs": (C.c_int64, [_I, _PI, _PI, _PI, _PI]),
    "song2_bispectra_create": (_I, [_P, C.POINTER(BispectraSpec), C.POINTER(_P), C.c_char_p]),
    "song2_bispectra_destroy": (None, [_P]),
    "song2_bispectra_size": (C.c_int64, [_P]),
    "song2_bispectra_run": (_I, [_P, _P, _P, _P, C.c_char_p]),
    "song2_bispectra_last_ms": (C.c_float, [_P]),
    "song2_gpu_bispectra": (_I, [C.POINTER(Spec), C.POINTER(LosSpec), C.POINTER(BispectraSpec), _PD, _PD,
                                 C.c_char_p]),
    "song2_bispectra_add_quadratic": (None, [_PD, _PD, C.c_int64, _I]),
}


# callback types of the table providers (song2_fo_provider, song2_bg_provider)
FO_PROVIDER = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_double))
BG_PROVIDER = C.CFUNCTYPE(C.c_int, C.c_void_p, C.c_double, C.POINTER(C.c_double))


def bind(lib, host_only=False):
    """Set the ctypes signatures of the entry points; host_only binds just the
    host-side functions that a library exports (a CPU-only build of the input
    provider, which carries no GPU entry points)."""
    for name, (res, args) in SIGNATURES.items():
        if host_only and ("_ctx_" in name or "_gpu_" in name or "_los_" in name or name == "song2_autotune"):
            continue
        try:
            f = getattr(lib, name)
        except AttributeError:
            if host_only:
                continue
            raise
        f.restype = res
        f.argtypes = args
    return lib


_lib = None


def load(path=None):
    """Load the in-tree product library (build it with song_gb300.build.build()).
    SONG2_LIB names another build of the same library (the phase-timer build of
    song_gb300.build, for instance)."""
    global _lib
    if path is None:
        path = os.environ.get("SONG2_LIB") or LIB_PATH
    if _lib is None:
        if not os.path.exists(path):
            raise RuntimeError(f"song2 library not built: {path} is missing (run song_gb300.build.build())")
        _lib = bind(C.CDLL(path))
    return _lib


def dptr(a):
    assert a.dtype == np.float64 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_PD)


def iptr(a):
    assert a.dtype == np.int32 and a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(_PI)


def errbuf():
    return C.create_string_buffer(SONG2_ERRLEN)

"""ctypes mirror of include/climaland_cuda.h.

Constants and structures here follow the C header one-to-one; the header is
the source of truth for the ABI.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

# status codes
CLM_OK = 0
CLM_ERR_ARG = 1
CLM_ERR_CUDA = 2
CLM_ERR_TIMEOUT = 3
CLM_ERR_NAN = 4
CLM_ERR_STATE = 5
CLM_ERR_UNSUPPORTED = 6

STATUS_NAMES = {
    0: "CLM_OK",
    1: "CLM_ERR_ARG",
    2: "CLM_ERR_CUDA",
    3: "CLM_ERR_TIMEOUT",
    4: "CLM_ERR_NAN",
    5: "CLM_ERR_STATE",
    6: "CLM_ERR_UNSUPPORTED",
}

# per-column flags
CLM_COL_NONFINITE = 0x1
CLM_COL_DIVERGED = 0x2
CLM_COL_NOT_CONVERGED = 0x4
CLM_COL_GUESS_FALLBACK = 0x8
CLM_COL_PSI_POSITIVE = 0x10

# enums
CLM_MODEL_RICHARDS = 0
CLM_MODEL_ENERGY_HYDROLOGY = 1
CLM_PREC_FP64 = 0
CLM_PREC_MIXED = 1
CLM_NEWTON_FIXED = 0
CLM_NEWTON_TOL = 1
CLM_GUESS_NONE = 0
CLM_GUESS_NETWORK = 1
CLM_GUESS_EXTRAPOLATE = 2
CLM_SCHED_STATIC = 0
CLM_SCHED_DYNAMIC = 1
CLM_TOL_TILES = 0
CLM_TOL_REGROUP = 1
CLM_TOL_SPLIT = 2
CLM_TOL_AUTO = 3
CLM_BC_FLUX = 0
CLM_BC_FREE_DRAINAGE = 1
CLM_BC_STATE = 2
CLM_BC_FLUX_ADVECTIVE = 3
CLM_BC_PRECIP_RUNOFF = 4
CLM_BC_ATMOS = 5
CLM_RUNOFF_NONE = 0
CLM_RUNOFF_SURFACE = 1
CLM_RUNOFF_TOPMODEL = 2
CLM_RX_PSI_CANOPY = 0
CLM_RX_LAI = 1
CLM_RX_RAI = 2
CLM_RX_HEIGHT = 3
CLM_RX_ROOT_DEPTH = 4
CLM_RX_K_SAT = 5
CLM_RX_PSI63 = 6
CLM_RX_WEIBULL_C = 7
CLM_RX_NFIELDS = 8

# clm_atmos_field: rows of clm_set_atmos
ATMOS_FIELDS = ("P_LIQ", "T_AIR", "U_AIR", "Q_AIR", "P_AIR", "SW_D", "LW_D", "H_AIR", "GUSTINESS",
                "PAR_ALBEDO_DRY", "NIR_ALBEDO_DRY", "PAR_ALBEDO_WET", "NIR_ALBEDO_WET",
                "ALBEDO_TOP_THICKNESS", "EMISSIVITY", "Z_0M", "Z_0B", "D_DS", "EVAP_P", "EVAP_ALPHA")
for _i, _n in enumerate(ATMOS_FIELDS):
    globals()["CLM_AT_" + _n] = _i
CLM_AT_NFIELDS = len(ATMOS_FIELDS)

# clm_atmos_flux: rows of clm_atmos_fluxes
ATMOS_FLUXES = ("LHF", "SHF", "VAPOR_LIQ", "VAPOR_ICE", "R_N", "Q_SFC", "TOP_WATER", "TOP_HEAT")
for _i, _n in enumerate(ATMOS_FLUXES):
    globals()["CLM_AF_" + _n] = _i
CLM_AF_NFIELDS = len(ATMOS_FLUXES)
CLM_CM_VAN_GENUCHTEN = 0
CLM_CM_BROOKS_COREY = 1

CLM_P_NU = 0
CLM_P_K_SAT = 1
CLM_P_S_S = 2
CLM_P_THETA_R = 3
CLM_P_VG_ALPHA = 4
CLM_P_VG_N = 5
CLM_P_BC_PSI_B = 4
CLM_P_BC_C = 5
CLM_NPARAM_RICHARDS = 6
CLM_P_KAPPA_DRY = 6
CLM_P_KAPPA_SAT_FROZEN = 7
CLM_P_KAPPA_SAT_UNFROZEN = 8
CLM_P_RHOC_DS = 9
CLM_P_NU_SS_OM = 10
CLM_P_NU_SS_QUARTZ = 11
CLM_P_NU_SS_GRAVEL = 12
CLM_NPARAM_EH = 13
CLM_P_F_MAX = 13
CLM_P_F_OVER = 14
CLM_P_R_SB = 15
CLM_NPARAM_MAX = 16

CLM_F_BASE = 0
CLM_F_AMP = 1
CLM_F_OMEGA = 2
CLM_F_PHASE = 3
CLM_F_PULSE_AMP = 4
CLM_F_PULSE_PERIOD = 5
CLM_F_PULSE_DUTY = 6
CLM_F_T_ADV = 7
CLM_F_NFIELDS = 8

CLM_BC_TOP_WATER = 0
CLM_BC_TOP_HEAT = 1
CLM_BC_BOTTOM_WATER = 2
CLM_BC_BOTTOM_HEAT = 3


class ClmEarthParams(ctypes.Structure):
    _fields_ = [
        ("rho_l", ctypes.c_double),
        ("rho_i", ctypes.c_double),
        ("cp_l", ctypes.c_double),
        ("cp_i", ctypes.c_double),
        ("T_0", ctypes.c_double),
        ("T_freeze", ctypes.c_double),
        ("LH_f0", ctypes.c_double),
        ("grav", ctypes.c_double),
    ]


class ClmAtmosParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in (
        "stefan", "gas_constant", "molmass_dryair", "molmass_water", "D_vapor", "LH_v0", "LH_s0",
        "cp_d", "cp_v", "T_triple", "press_triple", "von_karman", "Pr_0", "a_m", "a_h", "b_m", "b_h",
        "zeta_max")] + [("iterations", ctypes.c_int32), ("universal_functions", ctypes.c_int32),
                        ("gryanik_b_m", ctypes.c_double), ("gryanik_b_h", ctypes.c_double)]


# Python twin of clm_atmos_params_default (ClimaParams values; Gryanik et al.
# 2020 on the stable side, Businger-Dyer on the unstable side).
DEFAULT_ATMOS = dict(
    stefan=5.670374419e-8, gas_constant=8.3144598, molmass_dryair=0.02897,
    molmass_water=0.01801528, D_vapor=2.5e-5, LH_v0=2500800.0, LH_s0=2834400.0, cp_d=1004.5,
    cp_v=1859.0, T_triple=273.16, press_triple=611.657, von_karman=0.4, Pr_0=0.98, a_m=5.0,
    a_h=5.0, b_m=15.0, b_h=9.0, zeta_max=100.0, iterations=8, universal_functions=1,
    gryanik_b_m=0.3, gryanik_b_h=0.4,
)
# Businger-Dyer on both sides (CLM_UF_BUSINGER): Businger et al. (1971)
BUSINGER_ATMOS = dict(DEFAULT_ATMOS, Pr_0=0.74, a_m=4.7, a_h=4.7, universal_functions=0,
                      gryanik_b_m=0.0, gryanik_b_h=0.0)


# enum clm_universal_functions
CLM_UF_BUSINGER = 0
CLM_UF_GRYANIK = 1


def default_atmos_params() -> "ClmAtmosParams":
    a = ClmAtmosParams()
    for k, v in DEFAULT_ATMOS.items():
        setattr(a, k, v)
    return a


class ClmConfig(ctypes.Structure):
    _fields_ = [
        ("model", ctypes.c_int32),
        ("ncol", ctypes.c_int32),
        ("nlayers", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("newton_mode", ctypes.c_int32),
        ("max_iters", ctypes.c_int32),
        ("newton_tol", ctypes.c_double),
        ("energy_norm_scale", ctypes.c_double),
        ("learned_guess", ctypes.c_int32),
        ("bc_top_water", ctypes.c_int32),
        ("bc_top_heat", ctypes.c_int32),
        ("bc_bottom_water", ctypes.c_int32),
        ("bc_bottom_heat", ctypes.c_int32),
        ("kersten_alpha", ctypes.c_double),
        ("kersten_beta", ctypes.c_double),
        ("ice_impedance_omega", ctypes.c_double),
        ("visc_gamma", ctypes.c_double),
        ("visc_gamma_T_ref", ctypes.c_double),
        ("earth", ClmEarthParams),
        ("phase_change", ctypes.c_int32),
        ("pad0", ctypes.c_int32),
        ("forcing_seed", ctypes.c_uint64),
        ("cols_per_cta", ctypes.c_int32),
        ("schedule", ctypes.c_int32),
        ("graph", ctypes.c_int32),
        ("hydrology_cm", ctypes.c_int32),
        ("column_offset", ctypes.c_int64),
        ("host_chunks", ctypes.c_int32),
        ("runoff", ctypes.c_int32),
        ("tol_regroup", ctypes.c_int32),
        ("pad1", ctypes.c_int32),
    ]


# ClimaParams defaults for the LandParameters fields used on this path
# (density_liquid_water, density_ice_water, isobaric_specific_heat_liquid,
# isobaric_specific_heat_ice, thermodynamics_temperature_reference,
# temperature_water_freeze, latent_heat_sublimation_at_reference -
# latent_heat_vaporization_at_reference, gravitational_acceleration).
DEFAULT_EARTH = dict(
    rho_l=1000.0,
    rho_i=916.7,
    cp_l=4181.0,
    cp_i=2100.0,
    T_0=273.16,
    T_freeze=273.15,
    LH_f0=2834400.0 - 2500800.0,
    grav=9.81,
)


def default_config() -> ClmConfig:
    """Python twin of clm_config_default (usable without the CUDA library)."""
    c = ClmConfig()
    c.model = CLM_MODEL_ENERGY_HYDROLOGY
    c.ncol = 0
    c.nlayers = 0
    c.precision = CLM_PREC_FP64
    c.newton_mode = CLM_NEWTON_FIXED
    c.max_iters = 3
    c.newton_tol = 1e-8
    c.energy_norm_scale = 1.0
    c.learned_guess = 0
    c.bc_top_water = CLM_BC_FLUX
    c.bc_top_heat = CLM_BC_FLUX
    c.bc_bottom_water = CLM_BC_FREE_DRAINAGE
    c.bc_bottom_heat = CLM_BC_FREE_DRAINAGE
    c.kersten_alpha = 0.24
    c.kersten_beta = 18.3
    c.ice_impedance_omega = 7.0
    c.visc_gamma = 2.64e-2
    c.visc_gamma_T_ref = 288.0
    for k, v in DEFAULT_EARTH.items():
        setattr(c.earth, k, v)
    c.phase_change = 1
    c.forcing_seed = 0
    c.cols_per_cta = 0
    c.schedule = CLM_SCHED_STATIC
    c.graph = 0
    c.tol_regroup = CLM_TOL_AUTO
    return c


class ClmTuneEntry(ctypes.Structure):
    _fields_ = [
        ("cols_per_cta", ctypes.c_int32),
        ("schedule", ctypes.c_int32),
        ("grid", ctypes.c_int32),
        ("chosen", ctypes.c_int32),
        ("ms_per_step", ctypes.c_double),
    ]


def config_to_dict(c: ClmConfig) -> dict:
    out = {}
    for name, _ in ClmConfig._fields_:
        v = getattr(c, name)
        if name == "earth":
            v = {k: getattr(v, k) for k, _ in ClmEarthParams._fields_}
        elif name == "reserved":
            continue
        out[name] = v
    return out


PACKAGE_DIR = Path(__file__).resolve().parent
LIB_NAME = "libclimaland_cuda.so"


def library_path() -> Path:
    env = os.environ.get("CLIMALAND_CUDA_LIB")
    if env:
        return Path(env)
    return PACKAGE_DIR / "_build" / LIB_NAME


_DP = ctypes.POINTER(ctypes.c_double)
_IP = ctypes.POINTER(ctypes.c_int32)
_UP = ctypes.POINTER(ctypes.c_uint32)
_H = ctypes.c_void_p

# (name, restype, argtypes) for every symbol declared in the header.
SIGNATURES = [
    ("clm_config_default", None, [ctypes.POINTER(ClmConfig)]),
    ("clm_create", ctypes.c_int, [ctypes.POINTER(ClmConfig), ctypes.POINTER(_H)]),
    ("clm_destroy", None, [_H]),
    ("clm_last_error", ctypes.c_char_p, [_H]),
    ("clm_set_geometry", ctypes.c_int, [_H, _DP, _DP, _IP]),
    ("clm_set_faces", ctypes.c_int, [_H, _DP]),
    ("clm_set_params", ctypes.c_int, [_H, _DP, ctypes.c_int32]),
    ("clm_set_root_extraction", ctypes.c_int, [_H, _DP, ctypes.c_int32]),
    ("clm_atmos_params_default", None, [ctypes.POINTER(ClmAtmosParams)]),
    ("clm_set_atmos", ctypes.c_int, [_H, ctypes.POINTER(ClmAtmosParams), _DP, ctypes.c_int32]),
    ("clm_atmos_fluxes", ctypes.c_int, [_H, _DP, ctypes.c_int32]),
    ("clm_set_bc", ctypes.c_int, [_H, ctypes.c_int32, _DP, ctypes.c_int32]),
    ("clm_set_state", ctypes.c_int, [_H, _DP, _DP, _DP, _DP, _DP]),
    ("clm_get_state", ctypes.c_int, [_H, _DP, _DP, _DP, _DP, _DP]),
    ("clm_set_state_device", ctypes.c_int, [_H, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("clm_get_state_device", ctypes.c_int, [_H, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    ("clm_step", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_double, ctypes.c_int32]),
    ("clm_step_async", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_double, ctypes.c_int32]),
    ("clm_sync", ctypes.c_int, [_H]),
    ("clm_set_stream", ctypes.c_int, [_H, ctypes.c_void_p]),
    ("clm_step_host", ctypes.c_int, [_H, _DP, _DP, _DP, _DP, _DP, ctypes.c_double, ctypes.c_double,
                                     ctypes.c_int32]),
    ("clm_autotune", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_double, ctypes.c_int32,
                                    ctypes.c_void_p, ctypes.c_int32, _IP]),
    ("clm_get_launch_config", ctypes.c_int, [_H, _IP, _IP, _IP]),
    ("clm_get_budgets", ctypes.c_int, [_H, _DP, _DP]),
    ("clm_get_status", ctypes.c_int, [_H, _UP, _IP]),
    ("clm_update_aux", ctypes.c_int, [_H, ctypes.c_double, _DP, _DP, _DP, _DP, _DP, _DP, _DP]),
    ("clm_exp_tendency", ctypes.c_int, [_H, ctypes.c_double, _DP, _DP, _DP, _DP, _DP]),
    ("clm_imp_tendency", ctypes.c_int, [_H, ctypes.c_double, _DP, _DP, _DP, _DP, _DP]),
    ("clm_jacobian", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_double, _DP, _DP, _DP]),
    ("clm_solve", ctypes.c_int, [_H, _DP, _DP, _DP, _DP, _DP, _DP, _DP]),
    ("clm_load_mlp", ctypes.c_int, [_H, ctypes.c_void_p, ctypes.c_int64]),
    ("clm_features", ctypes.c_int, [_H, ctypes.c_double, ctypes.c_double, ctypes.c_void_p]),
    ("clm_mlp_create", ctypes.c_int, [ctypes.c_uint64, ctypes.POINTER(ctypes.c_void_p)]),
    ("clm_mlp_destroy", None, [ctypes.c_void_p]),
    ("clm_mlp_set_normalization", ctypes.c_int, [ctypes.c_void_p] + [ctypes.POINTER(ctypes.c_float)] * 4),
    ("clm_mlp_train", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
                                     ctypes.c_int32, ctypes.c_int32, ctypes.c_float,
                                     ctypes.POINTER(ctypes.c_float), ctypes.c_void_p]),
    ("clm_mlp_gradients", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)]),
    ("clm_mlp_predict", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                       ctypes.c_void_p]),
    ("clm_mlp_blob_bytes", ctypes.c_int64, []),
    ("clm_mlp_nparams", ctypes.c_int64, []),
    ("clm_mlp_get", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    ("clm_mlp_set", ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64]),
    ("clm_step_eh_noalloc", ctypes.c_int, [ctypes.POINTER(ClmConfig), ctypes.c_int32, ctypes.c_int32,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double,
                                           ctypes.c_double, ctypes.c_int32, ctypes.c_void_p]),
    ("clm_forcing_hash01", ctypes.c_double, [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int64]),
    ("clm_version", ctypes.c_char_p, []),
]


def declared_symbols() -> list[str]:
    return [s[0] for s in SIGNATURES]


def bind(lib: ctypes.CDLL) -> ctypes.CDLL:
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def dptr(a):
    """Pointer to a contiguous float64 numpy array, or NULL for None."""
    if a is None:
        return None
    return a.ctypes.data_as(_DP)


def iptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_IP)


def uptr(a):
    if a is None:
        return None
    return a.ctypes.data_as(_UP)

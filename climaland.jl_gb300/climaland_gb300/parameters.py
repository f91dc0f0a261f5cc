"""Soil parameter sets (host side).

Mirrors the reference's parameter constructors so that a caller builds the
same per-column values the Julia model would hold:
  - vanGenuchten (src/standalone/Soil/retention_models.jl:354-368)
  - RichardsParameters (src/standalone/Soil/rre.jl:7-48)
  - EnergyHydrologyParameters(toml_dict; ...) and its derived thermal
    parameters (src/standalone/Soil/energy_hydrology.jl:110-207,
    soil_heat_parameterizations.jl:338-392)
Values are numpy arrays (one entry per column) or scalars broadcast to all
columns.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _abi as A

# Soil thermal constants of the ClimaParams "Land" table used by
# EnergyHydrologyParameters (energy_hydrology.jl:132-145); the same values
# appear as in-test constants in test/standalone/Soil/soil_parameterizations.jl:39-56.
LAND_SOIL_CONSTANTS = dict(
    kappa_quartz=8.0,
    kappa_minerals=2.5,
    kappa_ice=2.21,
    kappa_liq=0.57,
    kappa_om=0.25,
    rho_p_quartz=2.66e3,
    rho_p_minerals=2.65e3,
    rho_p_om=1.3e3,
    rho_c_quartz=2.01e6,
    rho_c_om=2.51e6,
    rho_c_minerals=2.01e6,
    K_therm=2.4e-2,  # thermal_conductivity_of_air
)

# Scalar EnergyHydrology parameters (energy_hydrology.jl:174-180), pinned by
# test/standalone/Soil/soil_parameterizations.jl:71-75.
KERSTEN_ALPHA = 0.24
KERSTEN_BETA = 18.3
VISC_GAMMA = 2.64e-2
VISC_GAMMA_T_REF = 288.0
ICE_IMPEDANCE_OMEGA = 7.0


@dataclass
class vanGenuchten:
    """van Genuchten closure: alpha (1/m), n; m = 1 - 1/n and the critical
    saturation S_c = (1 + ((n - 1)/n)^(1 - 2n))^(-m)."""

    alpha: np.ndarray
    n: np.ndarray

    @property
    def m(self):
        return 1.0 - 1.0 / np.asarray(self.n, dtype=np.float64)

    @property
    def S_c(self):
        n = np.asarray(self.n, dtype=np.float64)
        return (1.0 + ((n - 1.0) / n) ** (1.0 - 2.0 * n)) ** (-self.m)


@dataclass
class BrooksCorey:
    """Brooks-Corey closure (retention_models.jl:47-67): c, psi_b (m, < 0)
    and the critical saturation S_c = (1 + 1/c)^(-c). Its rows go where the
    van Genuchten alpha and n go (CLM_P_BC_PSI_B, CLM_P_BC_C) with
    cfg.hydrology_cm = CLM_CM_BROOKS_COREY."""

    c: np.ndarray
    psib: np.ndarray

    @property
    def S_c(self):
        c = np.asarray(self.c, dtype=np.float64)
        return (1.0 + 1.0 / c) ** (-c)


def closure_rows(hcm):
    """(row 4, row 5, cfg.hydrology_cm) for a closure object."""
    if isinstance(hcm, BrooksCorey):
        return hcm.psib, hcm.c, A.CLM_CM_BROOKS_COREY
    return hcm.alpha, hcm.n, A.CLM_CM_VAN_GENUCHTEN


@dataclass
class RichardsParameters:
    nu: np.ndarray
    hydrology_cm: vanGenuchten | BrooksCorey
    K_sat: np.ndarray
    S_s: np.ndarray
    theta_r: np.ndarray

    def soa(self, ncol: int) -> np.ndarray:
        p = np.zeros((A.CLM_NPARAM_RICHARDS, ncol))
        p[A.CLM_P_NU] = self.nu
        p[A.CLM_P_K_SAT] = self.K_sat
        p[A.CLM_P_S_S] = self.S_s
        p[A.CLM_P_THETA_R] = self.theta_r
        p[A.CLM_P_VG_ALPHA], p[A.CLM_P_VG_N], _ = closure_rows(self.hydrology_cm)
        return p


def kappa_solid(nu_ss_om, nu_ss_quartz, kappa_om, kappa_quartz, kappa_minerals):
    return (kappa_om ** nu_ss_om * kappa_quartz ** nu_ss_quartz
            * kappa_minerals ** (1.0 - nu_ss_om - nu_ss_quartz))


def kappa_sat_frozen(ks, nu, kappa_ice):
    return ks ** (1.0 - nu) * kappa_ice ** nu


def kappa_sat_unfrozen(ks, nu, kappa_l):
    return ks ** (1.0 - nu) * kappa_l ** nu


def kappa_dry(rho_p, nu, ks, kappa_air, a=0.053):
    rho_b_dry = (1.0 - nu) * rho_p
    num = (a * ks - kappa_air) * rho_b_dry + kappa_air * rho_p
    den = rho_p - (1.0 - a) * rho_b_dry
    return num / den


@dataclass
class EnergyHydrologyParameters:
    kappa_dry: np.ndarray
    kappa_sat_frozen: np.ndarray
    kappa_sat_unfrozen: np.ndarray
    rho_c_ds: np.ndarray
    nu: np.ndarray
    nu_ss_om: np.ndarray
    nu_ss_quartz: np.ndarray
    nu_ss_gravel: np.ndarray
    hydrology_cm: vanGenuchten | BrooksCorey
    K_sat: np.ndarray
    S_s: np.ndarray
    theta_r: np.ndarray
    alpha: float = KERSTEN_ALPHA
    beta: float = KERSTEN_BETA
    Omega: float = ICE_IMPEDANCE_OMEGA
    gamma: float = VISC_GAMMA
    gamma_T_ref: float = VISC_GAMMA_T_REF

    @classmethod
    def from_composition(cls, *, nu, nu_ss_om, nu_ss_quartz, nu_ss_gravel,
                         hydrology_cm, K_sat, S_s, theta_r, constants=None, **kw):
        """The toml-dict constructor: derived rho_c_ds, kappa_dry,
        kappa_sat_frozen, kappa_sat_unfrozen from the soil composition."""
        c = dict(LAND_SOIL_CONSTANTS)
        if constants:
            c.update(constants)
        rest = 1.0 - nu_ss_om - nu_ss_quartz - nu_ss_gravel
        rho_p = (nu_ss_om * c["rho_p_om"] + nu_ss_quartz * c["rho_p_quartz"]
                 + nu_ss_gravel * c["rho_p_minerals"] + rest * c["rho_p_minerals"])
        rho_c_ss = (nu_ss_om * c["rho_c_om"] + nu_ss_quartz * c["rho_c_quartz"]
                    + nu_ss_gravel * c["rho_c_minerals"] + rest * c["rho_c_minerals"])
        rho_c_ds = (1.0 - nu) * rho_c_ss
        ks = kappa_solid(nu_ss_om, nu_ss_quartz, c["kappa_om"], c["kappa_quartz"], c["kappa_minerals"])
        return cls(
            kappa_dry=kappa_dry(rho_p, nu, ks, c["K_therm"]),
            kappa_sat_frozen=kappa_sat_frozen(ks, nu, c["kappa_ice"]),
            kappa_sat_unfrozen=kappa_sat_unfrozen(ks, nu, c["kappa_liq"]),
            rho_c_ds=rho_c_ds, nu=nu, nu_ss_om=nu_ss_om, nu_ss_quartz=nu_ss_quartz,
            nu_ss_gravel=nu_ss_gravel, hydrology_cm=hydrology_cm, K_sat=K_sat,
            S_s=S_s, theta_r=theta_r, **kw)

    def soa(self, ncol: int) -> np.ndarray:
        p = np.zeros((A.CLM_NPARAM_EH, ncol))
        p[A.CLM_P_NU] = self.nu
        p[A.CLM_P_K_SAT] = self.K_sat
        p[A.CLM_P_S_S] = self.S_s
        p[A.CLM_P_THETA_R] = self.theta_r
        p[A.CLM_P_VG_ALPHA], p[A.CLM_P_VG_N], _ = closure_rows(self.hydrology_cm)
        p[A.CLM_P_KAPPA_DRY] = self.kappa_dry
        p[A.CLM_P_KAPPA_SAT_FROZEN] = self.kappa_sat_frozen
        p[A.CLM_P_KAPPA_SAT_UNFROZEN] = self.kappa_sat_unfrozen
        p[A.CLM_P_RHOC_DS] = self.rho_c_ds
        p[A.CLM_P_NU_SS_OM] = self.nu_ss_om
        p[A.CLM_P_NU_SS_QUARTZ] = self.nu_ss_quartz
        p[A.CLM_P_NU_SS_GRAVEL] = self.nu_ss_gravel
        return p

    def apply_scalars(self, cfg: A.ClmConfig) -> None:
        cfg.kersten_alpha = self.alpha
        cfg.kersten_beta = self.beta
        cfg.ice_impedance_omega = self.Omega
        cfg.visc_gamma = self.gamma
        cfg.visc_gamma_T_ref = self.gamma_T_ref

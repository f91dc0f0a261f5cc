"""Seeded synthetic soil-column workloads.

The reference publishes no column-step dataset; these generators produce
inputs with the shapes, sizes and value ranges of the five benchmark
configurations (plain Richards 1024x20; plain EnergyHydrology 65,536x15;
uneven CSR columns 262,144 x U{4..30}; learned-guess evaluation
262,144x20; full scale 1,048,576x20) from numpy PCG64 generators with fixed
seeds. All arrays use the C ABI layout: cells column-contiguous with level 0
at the bottom, per-column parameter and forcing rows as SoA blocks.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _abi as A

# Reference-test constants for the derived frozen conductivity rule:
# kappa_sat_frozen / kappa_sat_unfrozen = (kappa_ice / kappa_liq) ** nu, which
# is what kappa_sat_frozen / kappa_sat_unfrozen
# (soil_heat_parameterizations.jl:359-373) give for a common solid
# conductivity; kappa_ice = 2.21, kappa_liq = 0.57
# (test/standalone/Soil/soil_parameterizations.jl:55-56).
KAPPA_ICE = 2.21
KAPPA_LIQ = 0.57

DAY = 86400.0


@dataclass
class Workload:
    """Everything a soil-column run needs, in C ABI layout."""

    name: str
    cfg: A.ClmConfig
    ncol: int
    offsets: np.ndarray  # int32, ncol + 1
    z_lo: np.ndarray
    z_hi: np.ndarray
    params: np.ndarray  # (nparams, ncol) float64
    forcing: dict  # slot -> (CLM_F_NFIELDS, ncol) float64
    vartheta_l: np.ndarray
    theta_i: np.ndarray | None
    rho_e_int: np.ndarray | None
    intF_w: np.ndarray
    intF_e: np.ndarray | None
    t0: float
    dt: float
    nsteps: int
    meta: dict = field(default_factory=dict)
    # root-extraction canopy values (CLM_RX_NFIELDS, ncol), or None
    root: np.ndarray | None = None
    # drivers of the atmosphere-driven top boundary (CLM_AT_NFIELDS, ncol)
    # and its constants (ClmAtmosParams; None: the defaults), or None
    atmos: np.ndarray | None = None
    atmos_params: object = None
    # face coordinates of stretched columns (ncells + ncol: column c's
    # n + 1 faces at offsets[c] + c ...), or None for uniform layers
    z_faces: np.ndarray | None = None

    @property
    def ncells(self) -> int:
        return int(self.offsets[-1])

    @property
    def nlayers(self) -> np.ndarray:
        return np.diff(self.offsets)

    def copy_state(self):
        def c(a):
            return None if a is None else a.copy()

        return (c(self.vartheta_l), c(self.theta_i), c(self.rho_e_int),
                c(self.intF_w), c(self.intF_e))

    def subset(self, ncol: int) -> "Workload":
        """First `ncol` columns (a bounded sample of the same workload)."""
        return self.columns(0, min(ncol, self.ncol), name=f"{self.name}[:{min(ncol, self.ncol)}]")

    def columns(self, c0: int, c1: int, name: str | None = None) -> "Workload":
        """Columns [c0, c1) as a workload of their own. Its config's
        column_offset keeps the global column indices (the rain-pulse hash),
        so stepping the parts gives the same bits as stepping the whole."""
        assert 0 <= c0 < c1 <= self.ncol
        a, b = int(self.offsets[c0]), int(self.offsets[c1])

        def cells(x):
            return None if x is None else x[a:b].copy()

        def cols(x):
            return None if x is None else x[c0:c1].copy()

        cfg = A.ClmConfig.from_buffer_copy(self.cfg)
        cfg.ncol = c1 - c0
        cfg.column_offset = self.cfg.column_offset + c0
        return Workload(
            name=name or f"{self.name}[{c0}:{c1}]", cfg=cfg, ncol=c1 - c0,
            offsets=(self.offsets[c0: c1 + 1] - a).astype(np.int32), z_lo=cols(self.z_lo),
            z_hi=cols(self.z_hi), params=np.ascontiguousarray(self.params[:, c0:c1]),
            forcing={k: np.ascontiguousarray(v[:, c0:c1]) for k, v in self.forcing.items()},
            vartheta_l=cells(self.vartheta_l), theta_i=cells(self.theta_i),
            rho_e_int=cells(self.rho_e_int), intF_w=cols(self.intF_w),
            intF_e=cols(self.intF_e), t0=self.t0, dt=self.dt,
            nsteps=self.nsteps, meta=dict(self.meta),
            root=None if self.root is None else np.ascontiguousarray(self.root[:, c0:c1]),
            atmos=None if self.atmos is None else np.ascontiguousarray(self.atmos[:, c0:c1]),
            atmos_params=self.atmos_params,
            z_faces=None if self.z_faces is None else self.z_faces[a + c0: b + c1].copy())


def _forcing(ncol: int) -> np.ndarray:
    return np.zeros((A.CLM_F_NFIELDS, ncol), dtype=np.float64)


def _hydraulics(rng: np.random.Generator, ncol: int) -> dict:
    """Per-column van Genuchten hydraulics shared by every configuration."""
    return dict(
        alpha=rng.uniform(0.5, 5.0, ncol),
        n=rng.uniform(1.2, 2.5, ncol),
        nu=rng.uniform(0.35, 0.55, ncol),
        theta_r=rng.uniform(0.02, 0.1, ncol),
        K_sat=10.0 ** rng.uniform(-7.0, -4.0, ncol),
        S_s=np.full(ncol, 1e-3),  # Soil.jl:351 default
    )


def _water_profile(rng, hyd, offsets, z_lo, z_hi):
    """vartheta_l per cell: a top value uniform in [theta_r + 0.05,
    nu - 0.05] with a linear depth gradient, clipped to the same range."""
    ncol = len(z_lo)
    lo = hyd["theta_r"] + 0.05
    hi = hyd["nu"] - 0.05
    top = rng.uniform(lo, hi)
    grad = rng.uniform(-0.05, 0.05, ncol)  # per metre of depth
    n = np.diff(offsets)
    col = np.repeat(np.arange(ncol), n)
    k = np.arange(offsets[-1]) - np.repeat(offsets[:-1], n)
    dz = (z_hi - z_lo) / n
    zc = z_lo[col] + (k + 0.5) * dz[col]
    depth = z_hi[col] - zc
    v = top[col] + grad[col] * depth
    return np.clip(v, lo[col], hi[col]), col, zc


def _frozen_equilibrium(theta_tot, T, hyd_c, earth):
    """theta_l = min(theta_star(T), theta_tot), theta_i from the remainder:
    the phase-change equilibrium of phase_change_source
    (soil_heat_parameterizations.jl:89-122) for a given liquid-equivalent
    water content theta_tot. hyd_c holds van Genuchten (alpha, n) or
    Brooks-Corey (psib, c) per cell."""
    nu, theta_r = hyd_c["nu"], hyd_c["theta_r"]
    bc = "psib" in hyd_c
    if bc:
        psib, c = hyd_c["psib"], hyd_c["c"]
    else:
        alpha, n = hyd_c["alpha"], hyd_c["n"]
        m = 1.0 - 1.0 / n
    rho_l, rho_i = earth["rho_l"], earth["rho_i"]
    LH_f0, grav, T_freeze = earth["LH_f0"], earth["grav"], earth["T_freeze"]
    sq = np.sqrt(np.finfo(np.float64).eps)
    tt = np.minimum(theta_tot, nu)
    S = (np.maximum(tt, theta_r + sq) - theta_r) / (np.maximum(nu, theta_r + sq) - theta_r)
    if bc:
        psi_w0 = psib * S ** (-1.0 / c)
    else:
        psi_w0 = -(((S ** (-1.0 / m) - 1.0) * alpha ** (-n)) ** (1.0 / n))
    Tf = np.maximum(T_freeze * np.exp(grav * psi_w0 / LH_f0), 1.0)
    H = (Tf - T > np.finfo(np.float64).eps).astype(np.float64)
    psi_T = LH_f0 / grav * np.log(T / Tf) * H
    if bc:
        S_star = ((psi_w0 + psi_T) / psib) ** (-c)
    else:
        S_star = (1.0 + (alpha * np.abs(psi_w0 + psi_T)) ** n) ** (-m)
    theta_star = S_star * (nu - theta_r) + theta_r
    theta_l = np.minimum(theta_star, theta_tot)
    theta_i = np.maximum(theta_tot - theta_l, 0.0) * rho_l / rho_i
    return theta_l, theta_i


def _rho_e(theta_l, theta_i, T, rhoc_ds, earth):
    rhoc = rhoc_ds + theta_l * earth["cp_l"] * earth["rho_l"] + theta_i * earth["cp_i"] * earth["rho_i"]
    return rhoc * (T - earth["T_0"]) - theta_i * earth["rho_i"] * earth["LH_f0"]


def _eh_params(rng, ncol, hyd):
    p = np.zeros((A.CLM_NPARAM_EH, ncol))
    p[A.CLM_P_NU] = hyd["nu"]
    p[A.CLM_P_K_SAT] = hyd["K_sat"]
    p[A.CLM_P_S_S] = hyd["S_s"]
    p[A.CLM_P_THETA_R] = hyd["theta_r"]
    p[A.CLM_P_VG_ALPHA] = hyd["alpha"]
    p[A.CLM_P_VG_N] = hyd["n"]
    p[A.CLM_P_RHOC_DS] = rng.uniform(1.5e6, 2.5e6, ncol)
    p[A.CLM_P_KAPPA_DRY] = rng.uniform(0.2, 0.4, ncol)
    ku = rng.uniform(1.5, 2.5, ncol)
    p[A.CLM_P_KAPPA_SAT_UNFROZEN] = ku
    p[A.CLM_P_KAPPA_SAT_FROZEN] = ku * (KAPPA_ICE / KAPPA_LIQ) ** hyd["nu"]
    p[A.CLM_P_NU_SS_OM] = 0.0
    p[A.CLM_P_NU_SS_QUARTZ] = rng.uniform(0.1, 0.9, ncol)
    p[A.CLM_P_NU_SS_GRAVEL] = 0.0
    return p


def _earth_dict(cfg):
    return {k: getattr(cfg.earth, k) for k, _ in A.ClmEarthParams._fields_}


def richards_c0(ncol: int = 1024, nlayers: int = 20, seed: int = 0) -> Workload:
    """Plain RichardsModel FP64: 1024 columns x 20 uniform layers over 2 m,
    flux top / free-drainage bottom, dt = 900 s, 3 Newton iterations, 96 steps."""
    rng = np.random.Generator(np.random.PCG64(1000 + seed))
    cfg = A.default_config()
    cfg.model = A.CLM_MODEL_RICHARDS
    cfg.ncol = ncol
    cfg.nlayers = nlayers
    cfg.bc_top_water = A.CLM_BC_FLUX
    cfg.bc_bottom_water = A.CLM_BC_FREE_DRAINAGE
    cfg.phase_change = 0
    hyd = _hydraulics(rng, ncol)
    offsets = (np.arange(ncol + 1) * nlayers).astype(np.int32)
    z_lo = np.full(ncol, -2.0)
    z_hi = np.zeros(ncol)
    v, _, _ = _water_profile(rng, hyd, offsets, z_lo, z_hi)
    params = np.zeros((A.CLM_NPARAM_RICHARDS, ncol))
    params[A.CLM_P_NU] = hyd["nu"]
    params[A.CLM_P_K_SAT] = hyd["K_sat"]
    params[A.CLM_P_S_S] = hyd["S_s"]
    params[A.CLM_P_THETA_R] = hyd["theta_r"]
    params[A.CLM_P_VG_ALPHA] = hyd["alpha"]
    params[A.CLM_P_VG_N] = hyd["n"]
    ftw = _forcing(ncol)
    ftw[A.CLM_F_BASE] = rng.uniform(-5e-7, 0.0, ncol)
    return Workload(
        name=f"richards_{ncol}x{nlayers}", cfg=cfg, ncol=ncol, offsets=offsets,
        z_lo=z_lo, z_hi=z_hi, params=params,
        forcing={A.CLM_BC_TOP_WATER: ftw}, vartheta_l=v, theta_i=None,
        rho_e_int=None, intF_w=np.zeros(ncol), intF_e=None, t0=0.0, dt=900.0,
        nsteps=96)


def _eh_common(rng, ncol, offsets, z_lo, z_hi, cfg, T_range=(265.0, 290.0)):
    earth = _earth_dict(cfg)
    hyd = _hydraulics(rng, ncol)
    params = _eh_params(rng, ncol, hyd)
    theta_tot, col, zc = _water_profile(rng, hyd, offsets, z_lo, z_hi)
    T_col = rng.uniform(*T_range, ncol)
    depth_frac = (z_hi[col] - zc) / (z_hi[col] - z_lo[col])
    T = T_col[col] + 2.0 * depth_frac  # slightly warmer at depth
    hyd_c = {k: hyd[k][col] for k in ("alpha", "n", "nu", "theta_r")}
    theta_l, theta_i = _frozen_equilibrium(theta_tot, T, hyd_c, earth)
    rho_e = _rho_e(theta_l, theta_i, T, params[A.CLM_P_RHOC_DS][col], earth)
    return hyd, params, theta_l, theta_i, rho_e


def energy_hydrology_c1(ncol: int = 65536, nlayers: int = 15, seed: int = 0) -> Workload:
    """Plain EnergyHydrology FP64: 65,536 columns x 15 layers over 3 m; top heat
    flux 150 sin(2 pi t / 86400) W/m^2 (positive upward) plus a constant water
    flux per column; EnergyWaterFreeDrainage bottom; dt = 450 s, 192 steps."""
    rng = np.random.Generator(np.random.PCG64(2000 + seed))
    cfg = A.default_config()
    cfg.model = A.CLM_MODEL_ENERGY_HYDROLOGY
    cfg.ncol = ncol
    cfg.nlayers = nlayers
    offsets = (np.arange(ncol + 1) * nlayers).astype(np.int32)
    z_lo = np.full(ncol, -3.0)
    z_hi = np.zeros(ncol)
    hyd, params, v, ti, e = _eh_common(rng, ncol, offsets, z_lo, z_hi, cfg)
    ftw = _forcing(ncol)
    ftw[A.CLM_F_BASE] = rng.uniform(-5e-7, 0.0, ncol)
    fth = _forcing(ncol)
    fth[A.CLM_F_AMP] = 150.0
    fth[A.CLM_F_OMEGA] = 2.0 * np.pi / DAY
    return Workload(
        name=f"energy_hydrology_{ncol}x{nlayers}", cfg=cfg, ncol=ncol,
        offsets=offsets, z_lo=z_lo, z_hi=z_hi, params=params,
        forcing={A.CLM_BC_TOP_WATER: ftw, A.CLM_BC_TOP_HEAT: fth},
        vartheta_l=v, theta_i=ti, rho_e_int=e, intF_w=np.zeros(ncol),
        intF_e=np.zeros(ncol), t0=0.0, dt=450.0, nsteps=192)


def uneven_c2(ncol: int = 262144, nmin: int = 4, nmax: int = 30, seed: int = 0) -> Workload:
    """Uneven EnergyHydrology columns: layer count uniform in {4..30}, bedrock
    depth uniform in [0.5, 5] m, CSR-packed; parameters and forcing as the
    65,536x15 configuration."""
    rng = np.random.Generator(np.random.PCG64(3000 + seed))
    cfg = A.default_config()
    cfg.model = A.CLM_MODEL_ENERGY_HYDROLOGY
    cfg.ncol = ncol
    cfg.nlayers = 0
    n = rng.integers(nmin, nmax + 1, ncol)
    offsets = np.zeros(ncol + 1, dtype=np.int32)
    offsets[1:] = np.cumsum(n)
    z_lo = -rng.uniform(0.5, 5.0, ncol)
    z_hi = np.zeros(ncol)
    hyd, params, v, ti, e = _eh_common(rng, ncol, offsets, z_lo, z_hi, cfg)
    ftw = _forcing(ncol)
    ftw[A.CLM_F_BASE] = rng.uniform(-5e-7, 0.0, ncol)
    fth = _forcing(ncol)
    fth[A.CLM_F_AMP] = 150.0
    fth[A.CLM_F_OMEGA] = 2.0 * np.pi / DAY
    return Workload(
        name=f"uneven_{ncol}x{nmin}-{nmax}", cfg=cfg, ncol=ncol, offsets=offsets,
        z_lo=z_lo, z_hi=z_hi, params=params,
        forcing={A.CLM_BC_TOP_WATER: ftw, A.CLM_BC_TOP_HEAT: fth},
        vartheta_l=v, theta_i=ti, rho_e_int=e, intF_w=np.zeros(ncol),
        intF_e=np.zeros(ncol), t0=0.0, dt=450.0, nsteps=192)


def full_scale_c4(ncol: int = 1048576, nlayers: int = 20, seed: int = 0) -> Workload:
    """Full scale: 1,048,576 EnergyHydrology columns x 20 layers, depth uniform
    in [1, 5] m, diurnal surface heat flux with amplitude U[100, 400] W/m^2,
    air temperature U[270, 300] K carried by infiltrating water, rain pulses
    of -1e-6 m/s on 10 % of hours (counter hash per column and hour),
    dt = 450 s, 8 days = 1536 steps."""
    rng = np.random.Generator(np.random.PCG64(4000 + seed))
    cfg = A.default_config()
    cfg.model = A.CLM_MODEL_ENERGY_HYDROLOGY
    cfg.ncol = ncol
    cfg.nlayers = nlayers
    cfg.bc_top_heat = A.CLM_BC_FLUX_ADVECTIVE
    cfg.forcing_seed = 4000 + seed
    offsets = (np.arange(ncol + 1) * nlayers).astype(np.int32)
    z_lo = -rng.uniform(1.0, 5.0, ncol)
    z_hi = np.zeros(ncol)
    hyd, params, v, ti, e = _eh_common(rng, ncol, offsets, z_lo, z_hi, cfg)
    ftw = _forcing(ncol)
    ftw[A.CLM_F_PULSE_AMP] = -1e-6
    ftw[A.CLM_F_PULSE_PERIOD] = 3600.0
    ftw[A.CLM_F_PULSE_DUTY] = 0.1
    fth = _forcing(ncol)
    fth[A.CLM_F_AMP] = rng.uniform(100.0, 400.0, ncol)
    fth[A.CLM_F_OMEGA] = 2.0 * np.pi / DAY
    fth[A.CLM_F_T_ADV] = rng.uniform(270.0, 300.0, ncol)
    return Workload(
        name=f"full_scale_{ncol}x{nlayers}", cfg=cfg, ncol=ncol,
        offsets=offsets, z_lo=z_lo, z_hi=z_hi, params=params,
        forcing={A.CLM_BC_TOP_WATER: ftw, A.CLM_BC_TOP_HEAT: fth},
        vartheta_l=v, theta_i=ti, rho_e_int=e, intF_w=np.zeros(ncol),
        intF_e=np.zeros(ncol), t0=0.0, dt=450.0, nsteps=1536)


def learned_eval_c3(ncol: int = 262144, nlayers: int = 20, seed: int = 0) -> Workload:
    """Learned-guess evaluation set: 262,144 EnergyHydrology columns x 20
    layers with the 65,536x15 configuration's distributions."""
    w = energy_hydrology_c1(ncol=ncol, nlayers=nlayers, seed=100 + seed)
    w.name = f"learned_eval_{ncol}x{nlayers}"
    return w


def richards_runoff(ncol: int = 1024, nlayers: int = 20, seed: int = 0,
                    runoff: int = A.CLM_RUNOFF_TOPMODEL) -> Workload:
    """RichardsModel driven by precipitation through a runoff model
    (RichardsAtmosDrivenFluxBC): the hydraulics of the 1024 x 20 Richards
    configuration over 2 m, water that rises from theta_r + 0.1 at the top to
    nu + 0.05 (saturated) at the bottom, no-flux bottom, precipitation
    -1e-6 + 5e-7 sin(2 pi t / day) m/s with hourly storms of -2e-5 m/s on 20 % of
    hours (heavier than most columns' K_sat), TOPMODEL f_max U[0.3, 0.7],
    f_over 3.28 1/m, R_sb 1.484e-7 m/s (the reference runoff tests' values),
    dt = 900 s."""
    rng = np.random.Generator(np.random.PCG64(7000 + seed))
    cfg = A.default_config()
    cfg.model = A.CLM_MODEL_RICHARDS
    cfg.ncol = ncol
    cfg.nlayers = nlayers
    cfg.bc_top_water = A.CLM_BC_PRECIP_RUNOFF
    cfg.bc_bottom_water = A.CLM_BC_FLUX
    cfg.runoff = runoff
    cfg.phase_change = 0
    cfg.forcing_seed = 7000 + seed
    hyd = _hydraulics(rng, ncol)
    offsets = (np.arange(ncol + 1) * nlayers).astype(np.int32)
    z_lo = np.full(ncol, -2.0)
    z_hi = np.zeros(ncol)
    frac = (np.arange(nlayers) + 0.5) / nlayers  # 0 at the bottom, 1 at the top
    lo = hyd["theta_r"][:, None] + 0.1
    hi = hyd["nu"][:, None] + 0.05
    v = (hi + (lo - hi) * frac[None, :]).ravel()
    params = np.zeros((A.CLM_NPARAM_MAX, ncol))
    params[A.CLM_P_NU] = hyd["nu"]
    params[A.CLM_P_K_SAT] = hyd["K_sat"]
    params[A.CLM_P_S_S] = hyd["S_s"]
    params[A.CLM_P_THETA_R] = hyd["theta_r"]
    params[A.CLM_P_VG_ALPHA] = hyd["alpha"]
    params[A.CLM_P_VG_N] = hyd["n"]
    params[A.CLM_P_F_MAX] = rng.uniform(0.3, 0.7, ncol)
    params[A.CLM_P_F_OVER] = 3.28
    params[A.CLM_P_R_SB] = 1.484e-4 / 1000.0
    ftw = _forcing(ncol)
    ftw[A.CLM_F_BASE] = -1e-6
    ftw[A.CLM_F_AMP] = 5e-7
    ftw[A.CLM_F_OMEGA] = 2.0 * np.pi / DAY
    ftw[A.CLM_F_PULSE_AMP] = -2e-5
    ftw[A.CLM_F_PULSE_PERIOD] = 3600.0
    ftw[A.CLM_F_PULSE_DUTY] = 0.2
    return Workload(
        name=f"richards_runoff_{ncol}x{nlayers}", cfg=cfg, ncol=ncol, offsets=offsets,
        z_lo=z_lo, z_hi=z_hi, params=params,
        forcing={A.CLM_BC_TOP_WATER: ftw}, vartheta_l=v, theta_i=None,
        rho_e_int=None, intF_w=np.zeros(ncol), intF_e=None, t0=0.0, dt=900.0,
        nsteps=96)


def brooks_corey(w: Workload, seed: int = 0) -> Workload:
    """The workload with a per-column Brooks-Corey closure instead of van
    Genuchten (cfg.hydrology_cm = CLM_CM_BROOKS_COREY): psi_b uniform in
    [-0.9, -0.05] m and c in [0.2, 0.6], around the reference's values
    (psi_b = -0.09, c = 0.228 in test/standalone/Soil/soil_parameterizations.jl:191;
    psi_b = -0.6, c = 0.43 in docs/src/tutorials/standalone/Soil/freezing_front.jl:106-108).
    EnergyHydrology states are re-partitioned into the Brooks-Corey freezing
    equilibrium at the same temperature and total water."""
    rng = np.random.Generator(np.random.PCG64(9000 + seed))
    cfg = A.ClmConfig.from_buffer_copy(w.cfg)
    cfg.hydrology_cm = A.CLM_CM_BROOKS_COREY
    params = w.params.copy()
    params[A.CLM_P_BC_PSI_B] = rng.uniform(-0.9, -0.05, w.ncol)
    params[A.CLM_P_BC_C] = rng.uniform(0.2, 0.6, w.ncol)
    v, ti, e = w.vartheta_l.copy(), None, None
    if cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY:
        earth = _earth_dict(cfg)
        col = np.repeat(np.arange(w.ncol), w.nlayers)
        rhoc_ds = params[A.CLM_P_RHOC_DS][col]
        rhoc = rhoc_ds + w.vartheta_l * earth["cp_l"] * earth["rho_l"] + w.theta_i * earth["cp_i"] * earth["rho_i"]
        T = earth["T_0"] + (w.rho_e_int + w.theta_i * earth["rho_i"] * earth["LH_f0"]) / rhoc
        theta_tot = w.vartheta_l + w.theta_i * earth["rho_i"] / earth["rho_l"]
        hyd_c = dict(psib=params[A.CLM_P_BC_PSI_B][col], c=params[A.CLM_P_BC_C][col],
                     nu=params[A.CLM_P_NU][col], theta_r=params[A.CLM_P_THETA_R][col])
        v, ti = _frozen_equilibrium(theta_tot, T, hyd_c, earth)
        e = _rho_e(v, ti, T, rhoc_ds, earth)
    return Workload(
        name=f"{w.name}_bc", cfg=cfg, ncol=w.ncol, offsets=w.offsets, z_lo=w.z_lo,
        z_hi=w.z_hi, params=params, forcing=w.forcing, vartheta_l=v, theta_i=ti,
        rho_e_int=e, intF_w=w.intF_w.copy(),
        intF_e=None if w.intF_e is None else w.intF_e.copy(), t0=w.t0, dt=w.dt,
        nsteps=w.nsteps, meta=dict(w.meta), root=None if w.root is None else w.root.copy(),
        atmos=None if w.atmos is None else w.atmos.copy(), atmos_params=w.atmos_params,
        z_faces=None if w.z_faces is None else w.z_faces.copy())


def with_root_extraction(w: Workload, seed: int = 0) -> Workload:
    """The EnergyHydrology workload with the RootExtraction source: per-column
    canopy values around the reference's plant-functional-type table
    (src/standalone/Vegetation/pfts.jl: K_sat_plant = 5e-9 m/s, psi63 =
    -4 MPa = -408 m, rooting depths 2-3.9 m): canopy psi U[-150, -10] m,
    LAI U[0.5, 5], RAI U[0.5, 3], height U[1, 20] m, rooting depth
    U[0.5, 4] m, K_sat_plant 10^U[-9, -8] m/s, psi63 U[-600, -200] m, Weibull
    c U[2, 5]."""
    assert w.cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY
    rng = np.random.Generator(np.random.PCG64(11000 + seed))
    r = np.zeros((A.CLM_RX_NFIELDS, w.ncol))
    r[A.CLM_RX_PSI_CANOPY] = rng.uniform(-150.0, -10.0, w.ncol)
    r[A.CLM_RX_LAI] = rng.uniform(0.5, 5.0, w.ncol)
    r[A.CLM_RX_RAI] = rng.uniform(0.5, 3.0, w.ncol)
    r[A.CLM_RX_HEIGHT] = rng.uniform(1.0, 20.0, w.ncol)
    r[A.CLM_RX_ROOT_DEPTH] = rng.uniform(0.5, 4.0, w.ncol)
    r[A.CLM_RX_K_SAT] = 10.0 ** rng.uniform(-9.0, -8.0, w.ncol)
    r[A.CLM_RX_PSI63] = rng.uniform(-600.0, -200.0, w.ncol)
    r[A.CLM_RX_WEIBULL_C] = rng.uniform(2.0, 5.0, w.ncol)
    out = w.columns(0, w.ncol, name=f"{w.name}_roots")
    out.root = r
    return out


def with_atmos(w: Workload, seed: int = 0, runoff: int = A.CLM_RUNOFF_NONE) -> Workload:
    """The EnergyHydrology workload under the atmosphere-driven top boundary
    (AtmosDrivenFluxBC, prescribed atmosphere and radiation, NoRunoff) with
    per-column drivers: air temperature within U[-8, 8] K of the top
    layer's temperature (the soil's own T_0 + (rho e + theta_i rho_i LH_f0) /
    rho c, so that frozen columns meet sub-freezing air), relative humidity
    U[0.2, 1], pressure U[80, 103] kPa, wind U[0.5, 10] m/s at U[2, 30] m,
    gustiness 1 m/s, liquid precipitation 0 (half the columns) or
    -U[1e-8, 5e-7] m/s, shortwave U[0, 900] W/m^2, longwave
    U[0.7, 1] sigma T_air^4; surface parameters: dry PAR / NIR albedo
    U[0.1, 0.3] / U[0.2, 0.45] and wet albedo U[0.5, 0.8] of the dry,
    albedo thickness U[0.01, 0.4] m (from the top layer alone to a mean over
    several), emissivity U[0.9, 1], z_0m U[1e-3, 5e-2] m, z_0b U[0.05, 1]
    z_0m, dry-layer depth U[0.01, 0.02] m, evaporation exponent U[1, 3] and
    scalar U[0.5, 2]. `runoff` selects the runoff model; TOPMODEL adds the
    parameter rows f_max U[0.2, 0.6], f_over U[2, 4] 1/m and R_sb U[0.5, 2]
    x 1.484e-7 m/s around the reference's defaults (Soil.jl:343-345: 3.28 and
    1.484e-4 / 1000)."""
    assert w.cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY
    rng = np.random.Generator(np.random.PCG64(12000 + seed))
    n = w.ncol
    d = np.zeros((A.CLM_AT_NFIELDS, n))
    e = w.cfg.earth
    top = w.offsets[1:].astype(np.int64) - 1
    ti = w.theta_i[top]
    nu = w.params[A.CLM_P_NU]
    tl = np.minimum(w.vartheta_l[top], nu - ti)
    rhoc = w.params[A.CLM_P_RHOC_DS] + tl * e.rho_l * e.cp_l + ti * e.rho_i * e.cp_i
    T_top = e.T_0 + (w.rho_e_int[top] + ti * e.rho_i * e.LH_f0) / rhoc
    T = T_top + rng.uniform(-8.0, 8.0, n)
    P = rng.uniform(80000.0, 103000.0, n)
    # Magnus saturation vapour pressure (Pa), only to place q below saturation
    e_s = 610.94 * np.exp(17.625 * (T - 273.15) / (T - 30.11))
    q_s = 0.622 * e_s / (P - 0.378 * e_s)
    d[A.CLM_AT_T_AIR] = T
    d[A.CLM_AT_P_AIR] = P
    d[A.CLM_AT_Q_AIR] = rng.uniform(0.2, 1.0, n) * q_s
    d[A.CLM_AT_U_AIR] = rng.uniform(0.5, 10.0, n)
    d[A.CLM_AT_H_AIR] = rng.uniform(2.0, 30.0, n)
    d[A.CLM_AT_GUSTINESS] = 1.0
    d[A.CLM_AT_P_LIQ] = np.where(rng.random(n) < 0.5, 0.0, -rng.uniform(1e-8, 5e-7, n))
    d[A.CLM_AT_SW_D] = rng.uniform(0.0, 900.0, n)
    d[A.CLM_AT_LW_D] = rng.uniform(0.7, 1.0, n) * 5.670374419e-8 * T ** 4
    par = rng.uniform(0.1, 0.3, n)
    nir = rng.uniform(0.2, 0.45, n)
    d[A.CLM_AT_PAR_ALBEDO_DRY] = par
    d[A.CLM_AT_NIR_ALBEDO_DRY] = nir
    d[A.CLM_AT_PAR_ALBEDO_WET] = par * rng.uniform(0.5, 0.8, n)
    d[A.CLM_AT_NIR_ALBEDO_WET] = nir * rng.uniform(0.5, 0.8, n)
    d[A.CLM_AT_ALBEDO_TOP_THICKNESS] = rng.uniform(0.01, 0.4, n)
    d[A.CLM_AT_EMISSIVITY] = rng.uniform(0.9, 1.0, n)
    z0m = 10.0 ** rng.uniform(-3.0, np.log10(5e-2), n)
    d[A.CLM_AT_Z_0M] = z0m
    d[A.CLM_AT_Z_0B] = z0m * rng.uniform(0.05, 1.0, n)
    d[A.CLM_AT_D_DS] = rng.uniform(0.01, 0.02, n)
    d[A.CLM_AT_EVAP_P] = rng.uniform(1.0, 3.0, n)
    d[A.CLM_AT_EVAP_ALPHA] = rng.uniform(0.5, 2.0, n)
    out = w.columns(0, w.ncol, name=f"{w.name}_atmos")
    out.cfg.bc_top_water = A.CLM_BC_ATMOS
    out.cfg.bc_top_heat = A.CLM_BC_ATMOS
    out.cfg.runoff = runoff
    if runoff == A.CLM_RUNOFF_TOPMODEL and out.params.shape[0] < A.CLM_NPARAM_MAX:
        prm = np.zeros((A.CLM_NPARAM_MAX, n))
        prm[: out.params.shape[0]] = out.params
        prm[A.CLM_P_F_MAX] = rng.uniform(0.2, 0.6, n)
        prm[A.CLM_P_F_OVER] = rng.uniform(2.0, 4.0, n)
        prm[A.CLM_P_R_SB] = 1.484e-7 * rng.uniform(0.5, 2.0, n)
        out.params = prm
    if runoff == A.CLM_RUNOFF_TOPMODEL:
        # a water table: in half the columns with K_sat < 2e-6 m/s (a table
        # under fast-draining soil empties within a step) the unfrozen layers
        # of the bottom third hold vartheta_l = nu + U[0, 0.002] without ice,
        # rho e_int re-derived at each layer's temperature
        nl = np.diff(out.offsets)
        col = np.repeat(np.arange(n), nl)
        k = np.arange(out.ncells) - np.repeat(out.offsets[:-1], nl)
        v, ti, re = out.vartheta_l.copy(), out.theta_i.copy(), out.rho_e_int.copy()
        nu_c = out.params[A.CLM_P_NU][col]
        rcds = out.params[A.CLM_P_RHOC_DS][col]
        tl0 = np.minimum(v, nu_c - ti)
        T = e.T_0 + (re + ti * e.rho_i * e.LH_f0) / (rcds + tl0 * e.rho_l * e.cp_l + ti * e.rho_i * e.cp_i)
        slow = (rng.random(n) < 0.5) & (out.params[A.CLM_P_K_SAT] < 2e-6)
        wet = slow[col] & (k < nl[col] // 3) & (T > e.T_freeze + 1.0)
        v[wet] = nu_c[wet] + rng.uniform(0.0, 0.002, int(wet.sum()))
        ti[wet] = 0.0
        tl = np.minimum(v, nu_c - ti)
        re[wet] = ((rcds + tl * e.rho_l * e.cp_l) * (T - e.T_0))[wet]
        out.vartheta_l, out.theta_i, out.rho_e_int = v, ti, re
    if runoff != A.CLM_RUNOFF_NONE:
        out.name = f"{out.name}_runoff{runoff}"
    out.forcing = {k: v for k, v in out.forcing.items()
                   if k not in (A.CLM_BC_TOP_WATER, A.CLM_BC_TOP_HEAT)}
    out.atmos = d
    return out


def generalized_exponential_faces(z_lo: float, z_hi: float, n: int, dz_bottom: float,
                                  dz_top: float) -> np.ndarray:
    """n + 1 face coordinates from z_lo to z_hi with a bottom layer of
    dz_bottom and a top layer of dz_top: a restatement of ClimaCore's
    GeneralizedExponentialStretching in the reverse mode that ClimaLand's
    Column and global domains use (src/shared_utilities/Domains.jl:198-207),
    i.e. measured from the surface down. With eta = j / n and the
    exponential map sigma(eta; h) = -h log(1 - (1 - exp(-1/h)) eta), the
    scale height h varies linearly in eta from h_s (fitted so that the first
    layer below the surface is dz_top) at eta = 1/n to h_d (fitted so that
    the deepest layer is dz_bottom) at eta = (n - 1)/n; face j lies at depth
    (z_hi - z_lo) sigma(eta_j; h(eta_j)). The library takes whatever faces
    the caller's mesh has, so this generator only shapes synthetic inputs."""
    depth = z_hi - z_lo
    a, b = dz_top / depth, dz_bottom / depth
    if not (n >= 3 and a < 1.0 / n < b < 1.0):
        raise ValueError("need dz_top < depth / n < dz_bottom < depth and n >= 3")

    def sigma(eta, h):
        return -h * np.log1p(-(-np.expm1(-1.0 / h)) * eta)

    def fit(fn, target):  # fn increasing in log h; bisection over log h
        lo, hi = -12.0, 12.0
        for _ in range(200):
            mid = 0.5 * (lo + hi)
            if fn(np.exp(mid)) < target:
                lo = mid
            else:
                hi = mid
        return np.exp(0.5 * (lo + hi))

    e1, en = 1.0 / n, (n - 1.0) / n
    h_s = fit(lambda h: sigma(e1, h), a)
    h_d = fit(lambda h: -(1.0 - sigma(en, h)), -b)
    eta = np.arange(n + 1) / n
    h = h_s + (h_d - h_s) * (eta - e1) / (en - e1)
    zeta = np.empty(n + 1)
    zeta[0] = 0.0
    zeta[n] = 1.0
    zeta[1:n] = sigma(eta[1:n], h[1:n])
    faces = z_hi - depth * zeta[::-1]
    faces[0], faces[n] = z_lo, z_hi
    if not np.all(np.diff(faces) > 0):
        raise ValueError("stretching does not give increasing faces")
    return faces


def stretched(w: Workload, dz_bottom_frac=(0.15, 0.3), dz_top_frac=(0.01, 0.04),
              dz_top_min: float = 0.05, seed: int = 0) -> Workload:
    """The workload on stretched columns: each column keeps its depth and
    layer count, with generalized exponential faces whose top layer is
    U[dz_top_frac] of the depth, at least dz_top_min metres (the reference's
    global domain has 0.05 m at the top and 10 m at the bottom of 50 m), and
    whose bottom layer is U[dz_bottom_frac] of it; a column too shallow for
    such a top layer keeps uniform faces. Thinner layers make the reference
    algorithm itself unstable at dt = 450 s: its explicit phase-change source
    overshoots when dt exceeds twice the thermal time 3 rho c dz^2 / kappa
    (about 6 minutes for a 1 cm layer), and three Newton iterations diverge on
    millimetre layers. The state arrays are kept cell by cell."""
    rng = np.random.Generator(np.random.PCG64(13000 + seed))
    nl = w.nlayers
    faces = np.empty(w.ncells + w.ncol)
    for c in range(w.ncol):
        n = int(nl[c])
        depth = w.z_hi[c] - w.z_lo[c]
        fb = rng.uniform(*dz_bottom_frac)
        ft = rng.uniform(*dz_top_frac)
        fb = max(fb, 1.5 / n)
        ft = max(ft, dz_top_min / depth)
        o = int(w.offsets[c]) + c
        if ft < 0.5 / n:
            faces[o: o + n + 1] = generalized_exponential_faces(w.z_lo[c], w.z_hi[c], n, fb * depth,
                                                                ft * depth)
        else:
            faces[o: o + n + 1] = w.z_lo[c] + (w.z_hi[c] - w.z_lo[c]) * (np.arange(n + 1) / n)
            faces[o + n] = w.z_hi[c]
    out = w.columns(0, w.ncol, name=f"{w.name}_stretched")
    out.z_faces = faces
    return out


def richards_benchmark(ncol: int = 65536, seed: int = 0) -> Workload:
    """The geometry and solver settings of the reference's RichardsModel GPU
    benchmark (experiments/benchmarks/richards.jl:64-137) on synthetic
    columns: 15 layers over 50 m stretched with dz_tuple = (10.0, 0.1)
    (global_domain, Domains.jl:1292-1298), RichardsModel{FT}(domain, forcing)
    defaults (Soil.jl:339-365): RichardsAtmosDrivenFluxBC with
    TOPMODELRunoff (f_over 3.28 1/m, R_sb 1.484e-7 m/s, f_max U[0.3, 0.7] in
    place of the topmodel_fmax map), no-flux bottom, S_s = 1e-3; dt = 1800 s,
    ARS111 with 2 Newton iterations, one week = 336 steps; the benchmark's
    hydrostatic initial profile (vartheta_l = nu + S_s (z_grad - z) below
    z_grad, van Genuchten saturation above) with the water table at
    z_grad = zmin / 5 = -10 m (the benchmark's z_grad = zmin / 5 + (zmax - zmin)
    / 2.5 = +10 m lies above the surface: every layer starts supersaturated,
    z_wt = depth - h_sat is about -4 m and TOPMODEL's R_sb exp(-f_over z_wt)
    drains ~0.3 m/s, after which the reference algorithm's states leave the
    physical range within tens of steps);
    precipitation -1e-6 + 5e-7 sin(2 pi t / day) m/s with hourly storms of
    -2e-5 m/s on 10 % of hours in place of the ERA5 rates; the hydraulics of
    the 1024 x 20 configuration."""
    rng = np.random.Generator(np.random.PCG64(14000 + seed))
    nlayers = 15
    cfg = A.default_config()
    cfg.model = A.CLM_MODEL_RICHARDS
    cfg.ncol = ncol
    cfg.nlayers = nlayers
    cfg.bc_top_water = A.CLM_BC_PRECIP_RUNOFF
    cfg.bc_bottom_water = A.CLM_BC_FLUX
    cfg.runoff = A.CLM_RUNOFF_TOPMODEL
    cfg.max_iters = 2
    cfg.phase_change = 0
    cfg.forcing_seed = 14000 + seed
    hyd = _hydraulics(rng, ncol)
    offsets = (np.arange(ncol + 1) * nlayers).astype(np.int32)
    zmin, zmax = -50.0, 0.0
    f1 = generalized_exponential_faces(zmin, zmax, nlayers, 10.0, 0.1)
    faces = np.tile(f1, ncol)
    zc = 0.5 * (f1[:-1] + f1[1:])
    z_grad = zmin / 5.0
    nu, tr = hyd["nu"][:, None], hyd["theta_r"][:, None]
    al, vn = hyd["alpha"][:, None], hyd["n"][:, None]
    m = 1.0 - 1.0 / vn
    z = zc[None, :]
    above = z > z_grad
    S = (1.0 + (al * np.abs(z - z_grad)) ** vn) ** (-m)
    v = np.where(above, S * (nu - tr) + tr, -hyd["S_s"][:, None] * (z - z_grad) + nu).ravel()
    params = np.zeros((A.CLM_NPARAM_MAX, ncol))
    params[A.CLM_P_NU] = hyd["nu"]
    params[A.CLM_P_K_SAT] = hyd["K_sat"]
    params[A.CLM_P_S_S] = hyd["S_s"]
    params[A.CLM_P_THETA_R] = hyd["theta_r"]
    params[A.CLM_P_VG_ALPHA] = hyd["alpha"]
    params[A.CLM_P_VG_N] = hyd["n"]
    params[A.CLM_P_F_MAX] = rng.uniform(0.3, 0.7, ncol)
    params[A.CLM_P_F_OVER] = 3.28
    params[A.CLM_P_R_SB] = 1.484e-4 / 1000.0
    ftw = _forcing(ncol)
    ftw[A.CLM_F_BASE] = -1e-6
    ftw[A.CLM_F_AMP] = 5e-7
    ftw[A.CLM_F_OMEGA] = 2.0 * np.pi / DAY
    ftw[A.CLM_F_PULSE_AMP] = -2e-5
    ftw[A.CLM_F_PULSE_PERIOD] = 3600.0
    ftw[A.CLM_F_PULSE_DUTY] = 0.1
    return Workload(
        name=f"richards_benchmark_{ncol}x{nlayers}_stretched", cfg=cfg, ncol=ncol,
        offsets=offsets, z_lo=np.full(ncol, zmin), z_hi=np.full(ncol, zmax), params=params,
        forcing={A.CLM_BC_TOP_WATER: ftw}, vartheta_l=v, theta_i=None, rho_e_int=None,
        intF_w=np.zeros(ncol), intF_e=None, t0=0.0, dt=1800.0, nsteps=336, z_faces=faces)


def global_eh_stretched(ncol: int = 65536, seed: int = 0) -> Workload:
    """EnergyHydrology on the reference's global soil column: 15 layers over
    50 m with global_domain's default dz_tuple = (10.0, 0.05)
    (Domains.jl:1292-1298), the 65,536 x 15 configuration's hydraulics,
    thermal parameters, initial temperatures and forcing."""
    w = energy_hydrology_c1(ncol=ncol, nlayers=15, seed=seed)
    f1 = generalized_exponential_faces(-50.0, 0.0, 15, 10.0, 0.05)
    out = w.columns(0, w.ncol, name=f"global_eh_{ncol}x15_stretched")
    out.z_lo = np.full(ncol, -50.0)
    out.z_hi = np.zeros(ncol)
    out.z_faces = np.tile(f1, ncol)
    return out


CONFIGS = {
    "c0": richards_c0,
    "c1": energy_hydrology_c1,
    "c2": uneven_c2,
    "c3": learned_eval_c3,
    "c4": full_scale_c4,
}


def make_workload(name, cfg, *, z_lo, z_hi, nlayers, params, forcing=None,
                  vartheta_l, theta_i=None, rho_e_int=None, intF_w=None,
                  intF_e=None, t0=0.0, dt=1.0, nsteps=1) -> Workload:
    """Assemble a Workload from explicit arrays (uniform or per-column layer
    counts). Scalars for z_lo / z_hi broadcast over columns."""
    params = np.ascontiguousarray(params, dtype=np.float64)
    ncol = params.shape[1]
    nl = np.broadcast_to(np.asarray(nlayers, dtype=np.int64), (ncol,))
    offsets = np.zeros(ncol + 1, dtype=np.int32)
    offsets[1:] = np.cumsum(nl)
    cfg = A.ClmConfig.from_buffer_copy(cfg)
    cfg.ncol = ncol
    cfg.nlayers = int(nl[0]) if np.all(nl == nl[0]) else 0
    eh = cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY
    nc = int(offsets[-1])

    def cells(a):
        if a is None:
            return None
        return np.ascontiguousarray(np.broadcast_to(np.asarray(a, dtype=np.float64), (nc,)))

    return Workload(
        name=name, cfg=cfg, ncol=ncol, offsets=offsets,
        z_lo=np.ascontiguousarray(np.broadcast_to(np.asarray(z_lo, float), (ncol,))),
        z_hi=np.ascontiguousarray(np.broadcast_to(np.asarray(z_hi, float), (ncol,))),
        params=params, forcing=dict(forcing or {}), vartheta_l=cells(vartheta_l),
        theta_i=cells(theta_i if theta_i is not None else (0.0 if eh else None)),
        rho_e_int=cells(rho_e_int) if eh else None,
        intF_w=np.zeros(ncol) if intF_w is None else np.asarray(intF_w, float).copy(),
        intF_e=(np.zeros(ncol) if intF_e is None else np.asarray(intF_e, float).copy()) if eh else None,
        t0=t0, dt=dt, nsteps=nsteps)


def constant_forcing(ncol: int, value) -> np.ndarray:
    f = _forcing(ncol)
    f[A.CLM_F_BASE] = value
    return f

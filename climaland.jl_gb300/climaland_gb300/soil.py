"""Host-side mirror of ClimaLand.Soil for the soil column step.

Same names and argument meaning as the reference types, for a batch of
independent columns:
  Column                      src/shared_utilities/Domains.jl:183-247
  RichardsModel               src/standalone/Soil/rre.jl:67-109
  EnergyHydrology             src/standalone/Soil/energy_hydrology.jl:226-271
  WaterFluxBC, HeatFluxBC, MoistureStateBC, TemperatureStateBC,
  FreeDrainage, EnergyWaterFreeDrainage, WaterHeatBC
                              src/standalone/Soil/boundary_conditions.jl:35-608
  PhaseChange                 energy_hydrology.jl:822-824
A boundary value is a number, a per-column array, or a `Forcing`
(the C ABI's forcing descriptor: base + amp sin(omega t + phase) + hashed
pulses), since the reference's Julia closures `bc(p, t)` cannot cross the ABI.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from . import _abi as A
from . import parameters as PR
from .workloads import Workload

# ---------------------------------------------------------------------------
# boundary values and conditions
# ---------------------------------------------------------------------------


@dataclass
class Forcing:
    """f(t) = base + amp sin(omega t + phase) + pulse_amp [hash(c, floor(t /
    pulse_period)) < pulse_duty]; every field a scalar or per-column array."""

    base: object = 0.0
    amp: object = 0.0
    omega: object = 0.0
    phase: object = 0.0
    pulse_amp: object = 0.0
    pulse_period: object = 0.0
    pulse_duty: object = 0.0
    T_adv: object = 0.0

    def soa(self, ncol: int) -> np.ndarray:
        f = np.zeros((A.CLM_F_NFIELDS, ncol))
        for i, name in enumerate(("base", "amp", "omega", "phase", "pulse_amp", "pulse_period",
                                  "pulse_duty", "T_adv")):
            f[i] = getattr(self, name)
        return f


def _forcing(value, ncol):
    if value is None:
        return None
    if isinstance(value, Forcing):
        return value.soa(ncol)
    return Forcing(base=np.broadcast_to(np.asarray(value, dtype=float), (ncol,))).soa(ncol)


@dataclass
class WaterFluxBC:
    flux: object

    kind = A.CLM_BC_FLUX


@dataclass
class HeatFluxBC:
    flux: object
    advected_temperature: object = None  # carries F_w rho e_liq(T) into the heat flux

    @property
    def kind(self):
        return A.CLM_BC_FLUX if self.advected_temperature is None else A.CLM_BC_FLUX_ADVECTIVE


@dataclass
class MoistureStateBC:
    vartheta_l: object

    kind = A.CLM_BC_STATE

    @property
    def flux(self):
        return self.vartheta_l


@dataclass
class TemperatureStateBC:
    T: object

    kind = A.CLM_BC_STATE

    @property
    def flux(self):
        return self.T


class FreeDrainage:
    kind = A.CLM_BC_FREE_DRAINAGE
    flux = None


class EnergyWaterFreeDrainage:
    kind = A.CLM_BC_FREE_DRAINAGE
    flux = None


@dataclass
class WaterHeatBC:
    water: object
    heat: object


@dataclass
class PhaseChange:
    explicit: bool = True


# ---------------------------------------------------------------------------
# domain and models
# ---------------------------------------------------------------------------


@dataclass
class Column:
    """A batch of `ncol` columns over zlim = (z_lo, z_hi) with `nelements`
    uniform layers each; zlim and nelements may be per-column arrays."""

    zlim: tuple
    nelements: object
    ncol: int = 1

    def arrays(self):
        z_lo = np.broadcast_to(np.asarray(self.zlim[0], float), (self.ncol,)).copy()
        z_hi = np.broadcast_to(np.asarray(self.zlim[1], float), (self.ncol,)).copy()
        n = np.broadcast_to(np.asarray(self.nelements, np.int64), (self.ncol,))
        offsets = np.zeros(self.ncol + 1, np.int32)
        offsets[1:] = np.cumsum(n)
        return z_lo, z_hi, offsets

    def centers(self):
        z_lo, z_hi, offsets = self.arrays()
        n = np.diff(offsets)
        col = np.repeat(np.arange(self.ncol), n)
        k = np.arange(offsets[-1]) - np.repeat(offsets[:-1], n)
        dz = (z_hi - z_lo) / n
        return z_lo[col] + (k + 0.5) * dz[col]


@dataclass
class RichardsModel:
    parameters: PR.RichardsParameters
    domain: Column
    boundary_conditions: dict
    sources: tuple = ()
    lateral_flow: bool = False

    model_kind = A.CLM_MODEL_RICHARDS

    def __post_init__(self):
        assert not self.lateral_flow  # rre.jl:106

    def prognostic_vars(self):
        return ("vartheta_l", "intF_vol_liq_water_dt")

    def initialize(self):
        z_lo, z_hi, offsets = self.domain.arrays()
        nc = int(offsets[-1])
        return dict(vartheta_l=np.zeros(nc), intF_w=np.zeros(self.domain.ncol))

    def config(self) -> A.ClmConfig:
        cfg = A.default_config()
        cfg.model = A.CLM_MODEL_RICHARDS
        cfg.phase_change = 0
        cfg.hydrology_cm = PR.closure_rows(self.parameters.hydrology_cm)[2]
        top, bot = self.boundary_conditions["top"], self.boundary_conditions["bottom"]
        cfg.bc_top_water = top.kind
        cfg.bc_bottom_water = bot.kind
        return cfg

    def forcing(self):
        ncol = self.domain.ncol
        top, bot = self.boundary_conditions["top"], self.boundary_conditions["bottom"]
        out = {}
        for slot, bc in ((A.CLM_BC_TOP_WATER, top), (A.CLM_BC_BOTTOM_WATER, bot)):
            f = _forcing(bc.flux, ncol)
            if f is not None:
                out[slot] = f
        return out

    def params_soa(self):
        return self.parameters.soa(self.domain.ncol)


@dataclass
class EnergyHydrology:
    parameters: PR.EnergyHydrologyParameters
    domain: Column
    boundary_conditions: dict
    sources: tuple = (PhaseChange(),)
    lateral_flow: bool = False
    earth: dict = field(default_factory=lambda: dict(A.DEFAULT_EARTH))

    model_kind = A.CLM_MODEL_ENERGY_HYDROLOGY

    def __post_init__(self):
        assert not self.lateral_flow  # energy_hydrology.jl:258

    def prognostic_vars(self):
        return ("vartheta_l", "theta_i", "rho_e_int", "intF_vol_liq_water_dt", "intF_e_dt")

    def initialize(self):
        z_lo, z_hi, offsets = self.domain.arrays()
        nc = int(offsets[-1])
        return dict(vartheta_l=np.zeros(nc), theta_i=np.zeros(nc), rho_e_int=np.zeros(nc),
                    intF_w=np.zeros(self.domain.ncol), intF_e=np.zeros(self.domain.ncol))

    def config(self) -> A.ClmConfig:
        cfg = A.default_config()
        cfg.model = A.CLM_MODEL_ENERGY_HYDROLOGY
        cfg.phase_change = int(any(isinstance(s, PhaseChange) for s in self.sources))
        cfg.hydrology_cm = PR.closure_rows(self.parameters.hydrology_cm)[2]
        for k, v in self.earth.items():
            setattr(cfg.earth, k, v)
        self.parameters.apply_scalars(cfg)
        top, bot = self.boundary_conditions["top"], self.boundary_conditions["bottom"]
        if isinstance(top, WaterHeatBC):
            cfg.bc_top_water, cfg.bc_top_heat = top.water.kind, top.heat.kind
        else:
            raise ValueError("top boundary must be a WaterHeatBC")
        if isinstance(bot, EnergyWaterFreeDrainage):
            cfg.bc_bottom_water = cfg.bc_bottom_heat = A.CLM_BC_FREE_DRAINAGE
        elif isinstance(bot, WaterHeatBC):
            cfg.bc_bottom_water, cfg.bc_bottom_heat = bot.water.kind, bot.heat.kind
        else:
            raise ValueError("bottom boundary must be WaterHeatBC or EnergyWaterFreeDrainage")
        return cfg

    def forcing(self):
        ncol = self.domain.ncol
        top, bot = self.boundary_conditions["top"], self.boundary_conditions["bottom"]
        out = {}
        pairs = [(A.CLM_BC_TOP_WATER, top.water.flux), (A.CLM_BC_TOP_HEAT, top.heat.flux)]
        if isinstance(bot, WaterHeatBC):
            pairs += [(A.CLM_BC_BOTTOM_WATER, bot.water.flux), (A.CLM_BC_BOTTOM_HEAT, bot.heat.flux)]
        for slot, v in pairs:
            f = _forcing(v, ncol)
            if f is not None:
                out[slot] = f
        adv = getattr(top.heat, "advected_temperature", None)
        if adv is not None:
            out[A.CLM_BC_TOP_HEAT][A.CLM_F_T_ADV] = adv
        return out

    def params_soa(self):
        return self.parameters.soa(self.domain.ncol)


def to_workload(model, Y, t0=0.0, dt=1.0, nsteps=1, name="model") -> Workload:
    """The C-ABI description (geometry, SoA parameters, forcing, state) of a
    model and its prognostic state Y."""
    z_lo, z_hi, offsets = model.domain.arrays()
    cfg = model.config()
    cfg.ncol = model.domain.ncol
    n = np.diff(offsets)
    cfg.nlayers = int(n[0]) if np.all(n == n[0]) else 0
    eh = cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY
    return Workload(
        name=name, cfg=cfg, ncol=model.domain.ncol, offsets=offsets, z_lo=z_lo, z_hi=z_hi,
        params=model.params_soa(), forcing=model.forcing(),
        vartheta_l=np.ascontiguousarray(Y["vartheta_l"], float),
        theta_i=np.ascontiguousarray(Y["theta_i"], float) if eh else None,
        rho_e_int=np.ascontiguousarray(Y["rho_e_int"], float) if eh else None,
        intF_w=np.ascontiguousarray(Y["intF_w"], float),
        intF_e=np.ascontiguousarray(Y["intF_e"], float) if eh else None,
        t0=t0, dt=dt, nsteps=nsteps)

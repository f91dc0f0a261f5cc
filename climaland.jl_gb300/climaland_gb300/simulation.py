"""LandSimulation / step! / solve! for soil column models on the GPU.

Mirrors src/simulations/Simulations.jl:115-332 for a soil-only model: the
default timestepper is IMEX ARS111 with NewtonsMethod(max_iters = 3,
update_j = UpdateEvery(NewNewtonIteration)) (:127-135); `step` advances one
step (:312-314), `solve` runs to tf (:322-332). The step itself runs in
libclimaland_cuda (no CPU fallback).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import _abi as A
from .device import SoilColumns
from .soil import to_workload


@dataclass
class NewtonsMethod:
    max_iters: int = 3
    convergence_tol: float | None = None  # ConvergenceChecker(MaximumError(tol)) per column
    energy_norm_scale: float = 1.0


@dataclass
class IMEXAlgorithm:
    tableau: str = "ARS111"
    newtons_method: NewtonsMethod = None

    def __post_init__(self):
        if self.tableau != "ARS111":
            raise ValueError("only ARS111 is built")
        if self.newtons_method is None:
            self.newtons_method = NewtonsMethod()


def ARS111():
    return "ARS111"


class LandSimulation:
    """LandSimulation(t0, tf, dt, model; Y0, timestepper, precision)."""

    def __init__(self, t0, tf, dt, model, Y0, timestepper=None, precision="fp64", steps_per_call=1):
        self.t0, self.tf, self.dt = float(t0), float(tf), float(dt)
        self.t = self.t0
        self.model = model
        self.timestepper = timestepper or IMEXAlgorithm(ARS111(), NewtonsMethod(max_iters=3))
        nm = self.timestepper.newtons_method
        w = to_workload(model, Y0, t0=t0, dt=dt)
        kw = dict(max_iters=nm.max_iters,
                  precision=A.CLM_PREC_MIXED if precision == "mixed" else A.CLM_PREC_FP64)
        if nm.convergence_tol is not None:
            kw.update(newton_mode=A.CLM_NEWTON_TOL, newton_tol=nm.convergence_tol,
                      energy_norm_scale=nm.energy_norm_scale)
        self._cols = SoilColumns(w, **kw)
        self.steps_per_call = int(steps_per_call)

    def step(self):
        """step!(landsim): one ARS111 step of every column."""
        self._cols.step(self.t, self.dt, 1)
        self.t += self.dt

    def solve(self):
        """solve!(landsim): step until tf."""
        n = int(round((self.tf - self.t) / self.dt))
        while n > 0:
            k = min(n, max(self.steps_per_call, 1))
            self._cols.step(self.t, self.dt, k)
            self.t += k * self.dt
            n -= k

    @property
    def Y(self):
        v, ti, e, fw, fe = self._cols.get_state()
        out = dict(vartheta_l=v, intF_w=fw)
        if ti is not None:
            out.update(theta_i=ti, rho_e_int=e, intF_e=fe)
        return out

    def budgets(self):
        return self._cols.budgets()

    def status(self):
        return self._cols.status()

    def close(self):
        self._cols.close()

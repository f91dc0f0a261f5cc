"""ORACLE — test infrastructure only.

ctypes wrapper of the C FP64 restatement in oracle/clm_oracle.c. Imported by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg as the
checker; nothing in the product imports it.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

ORACLE_DIR = Path(__file__).resolve().parent
REPO = ORACLE_DIR.parent
sys.path.insert(0, str(REPO / "climaland.jl_gb300"))

from climaland_gb300 import _abi as A  # noqa: E402

LIB_PATH = ORACLE_DIR / "_build" / "libclm_oracle.so"


def build(force: bool = False) -> Path:
    """Compile the oracle with the committed Makefile (gcc, OpenMP)."""
    srcs = [ORACLE_DIR / "clm_oracle.c", ORACLE_DIR / "clm_oracle.h",
            REPO / "include" / "climaland_cuda.h"]
    if (not force and LIB_PATH.exists()
            and all(LIB_PATH.stat().st_mtime >= s.stat().st_mtime for s in srcs)):
        return LIB_PATH
    subprocess.run(["make", "-s", "-C", str(ORACLE_DIR)], check=True)
    return LIB_PATH


class _Problem(ctypes.Structure):
    _fields_ = [
        ("cfg", A.ClmConfig),
        ("ncol", ctypes.c_int32),
        ("offsets", ctypes.POINTER(ctypes.c_int32)),
        ("z_lo", ctypes.POINTER(ctypes.c_double)),
        ("z_hi", ctypes.POINTER(ctypes.c_double)),
        ("params", ctypes.POINTER(ctypes.c_double)),
        ("nparams", ctypes.c_int32),
        ("forcing", ctypes.POINTER(ctypes.c_double) * 4),
        ("nthreads", ctypes.c_int32),
        ("root", ctypes.POINTER(ctypes.c_double)),
        ("atmos", ctypes.POINTER(ctypes.c_double)),
        ("atm", A.ClmAtmosParams),
        ("z_faces", ctypes.POINTER(ctypes.c_double)),
    ]


_lib = None

_D = ctypes.c_double
_DP = ctypes.POINTER(ctypes.c_double)
_PP = ctypes.POINTER(_Problem)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(str(LIB_PATH))
        ip = ctypes.POINTER(ctypes.c_int)
        ep = ctypes.POINTER(A.ClmEarthParams)
        sig = {
            "clmo_volumetric_liquid_fraction": [_D] * 3,
            "clmo_effective_saturation": [_D] * 3,
            "clmo_matric_potential": [_D] * 4,
            "clmo_inverse_matric_potential": [_D] * 4 + [ip],
            "clmo_pressure_head": [_D] * 7,
            "clmo_dpsidvartheta": [_D] * 7,
            "clmo_hydraulic_conductivity": [_D] * 3,
            "clmo_bc_matric_potential": [_D] * 3,
            "clmo_bc_inverse_matric_potential": [_D] * 3 + [ip],
            "clmo_bc_pressure_head": [_D] * 6,
            "clmo_bc_dpsidvartheta": [_D] * 6,
            "clmo_bc_hydraulic_conductivity": [_D] * 3,
            "clmo_impedance_factor": [_D] * 2,
            "clmo_harmonic_mean": [_D] * 2,
            "clmo_plant_water_flux": [_D] * 6,
            "clmo_weibull_conductivity": [_D] * 4,
            "clmo_root_distribution": [_D] * 2,
            "clmo_viscosity_factor": [_D] * 3,
            "clmo_heaviside": [_D] * 2,
            "clmo_soil_Tf_depressed": [_D] * 12,
            "clmo_thermal_time": [_D] * 3,
            "clmo_phase_change_source": [_D] * 14 + [ip],
            "clmo_volumetric_heat_capacity": [_D] * 3 + [ep],
            "clmo_temperature_from_rho_e_int": [_D] * 3 + [ep],
            "clmo_volumetric_internal_energy": [_D] * 3 + [ep],
            "clmo_volumetric_internal_energy_liq": [_D] + [ep],
            "clmo_kappa_sat": [_D] * 4,
            "clmo_thermal_conductivity": [_D] * 3,
            "clmo_relative_saturation": [_D] * 3,
            "clmo_kersten_number": [_D] * 7,
            "clmo_kappa_solid": [_D] * 5,
            "clmo_kappa_sat_frozen": [_D] * 3,
            "clmo_kappa_sat_unfrozen": [_D] * 3,
            "clmo_kappa_dry": [_D] * 4,
            "clmo_dry_soil_layer_thickness": [_D] * 4,
            "clmo_soil_conductance": [_D] * 6,
        }
        for name, args in sig.items():
            f = getattr(L, name)
            f.restype = _D
            f.argtypes = args
        L.clm_forcing_hash01.restype = _D
        L.clm_forcing_hash01.argtypes = [ctypes.c_uint64, ctypes.c_uint64, ctypes.c_int64]
        L.clmo_forcing_value.restype = _D
        L.clmo_forcing_value.argtypes = [_DP, ctypes.c_int32, ctypes.c_int32, _D, ctypes.c_uint64,
                                         ctypes.c_int64]
        L.clmo_update_cache.restype = ctypes.c_int
        L.clmo_update_cache.argtypes = [_PP, _DP, _DP, _DP, _D] + [_DP] * 9
        for nm in ("clmo_exp_tendency", "clmo_imp_tendency"):
            f = getattr(L, nm)
            f.restype = ctypes.c_int
            f.argtypes = [_PP, _DP, _DP, _DP, _D] + [_DP] * 5
        L.clmo_jacobian.restype = ctypes.c_int
        L.clmo_jacobian.argtypes = [_PP, _DP, _DP, _DP, _D, _D, _DP, _DP, _DP]
        L.clmo_solve.restype = ctypes.c_int
        L.clmo_solve.argtypes = [_PP] + [_DP] * 7
        L.clmo_step.restype = ctypes.c_int
        L.clmo_step.argtypes = [_PP, _DP, _DP, _DP, _DP, _DP, _D, _D, ctypes.c_int32,
                                ctypes.POINTER(ctypes.c_uint32), ctypes.POINTER(ctypes.c_int32)]
        L.clmo_budgets.restype = ctypes.c_int
        L.clmo_budgets.argtypes = [_PP, _DP, _DP, _DP, _DP, _DP]
        apar = ctypes.POINTER(A.ClmAtmosParams)
        L.clmo_q_vap_saturation.restype = _D
        L.clmo_q_vap_saturation.argtypes = [_D, _D, ctypes.c_int, apar, ep]
        L.clmo_similarity.restype = ctypes.c_int
        L.clmo_similarity.argtypes = [apar] + [_D] * 7 + [_DP]
        for nm in ("clmo_businger_psi_m", "clmo_businger_psi_h", "clmo_gryanik_psi_m", "clmo_gryanik_psi_h"):
            f = getattr(L, nm)
            f.restype = _D
            f.argtypes = [_D, apar]
        L.clmo_atmos_params_default.restype = None
        L.clmo_atmos_params_default.argtypes = [apar]
        L.clmo_atmos_fluxes.restype = ctypes.c_int
        L.clmo_atmos_fluxes.argtypes = [_PP, _DP, _DP, _DP, _DP]
        L.clmo_runoff.restype = ctypes.c_int
        L.clmo_runoff.argtypes = [_PP, _DP, _D] + [_DP] * 4
        _lib = L
    return _lib


def earth(cfg=None):
    if cfg is None:
        cfg = A.default_config()
    e = A.ClmEarthParams()
    ctypes.memmove(ctypes.byref(e), ctypes.byref(cfg.earth), ctypes.sizeof(e))
    return e


class Oracle:
    """The oracle bound to one workload (arrays are referenced, not copied)."""

    def __init__(self, w, nthreads: int | None = None):
        self.w = w
        self._keep = []
        P = _Problem()
        ctypes.memmove(ctypes.byref(P.cfg), ctypes.byref(w.cfg), ctypes.sizeof(A.ClmConfig))
        P.ncol = w.ncol

        def keep(a, dt=np.float64):
            a = np.ascontiguousarray(a, dtype=dt)
            self._keep.append(a)
            return a

        P.offsets = keep(w.offsets, np.int32).ctypes.data_as(ctypes.POINTER(ctypes.c_int32))
        P.z_lo = A.dptr(keep(w.z_lo))
        P.z_hi = A.dptr(keep(w.z_hi))
        prm = keep(w.params)
        P.params = A.dptr(prm)
        P.nparams = prm.shape[0]
        for slot in range(4):
            f = w.forcing.get(slot)
            P.forcing[slot] = A.dptr(keep(f)) if f is not None else None
        P.nthreads = int(nthreads if nthreads else (os.cpu_count() or 1))
        root = getattr(w, "root", None)
        P.root = A.dptr(keep(root)) if root is not None else None
        atmos = getattr(w, "atmos", None)
        P.atmos = A.dptr(keep(atmos)) if atmos is not None else None
        atm = getattr(w, "atmos_params", None) or A.default_atmos_params()
        ctypes.memmove(ctypes.byref(P.atm), ctypes.byref(atm), ctypes.sizeof(A.ClmAtmosParams))
        zf = getattr(w, "z_faces", None)
        P.z_faces = A.dptr(keep(zf)) if zf is not None else None
        self.P = P
        self.eh = w.cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY

    def set_cfg(self, **kw):
        for k, v in kw.items():
            setattr(self.P.cfg, k, v)

    def _st(self, state):
        v, ti, e = state[:3]
        return A.dptr(v), A.dptr(ti if self.eh else None), A.dptr(e if self.eh else None)

    def step(self, state, t, dt, nsteps):
        """Advance state (tuple of 5 arrays, modified in place)."""
        v, ti, e, fw, fe = state
        flags = np.zeros(self.w.ncol, np.uint32)
        iters = np.zeros(self.w.ncol, np.int32)
        rc = lib().clmo_step(ctypes.byref(self.P), A.dptr(v), A.dptr(ti if self.eh else None),
                             A.dptr(e if self.eh else None), A.dptr(fw),
                             A.dptr(fe if self.eh else None), float(t), float(dt), int(nsteps),
                             A.uptr(flags), A.iptr(iters))
        return rc, flags, iters

    def atmos_fluxes(self, state):
        """CLM_AF_NFIELDS x ncol diagnostics of the atmosphere-driven boundary."""
        out = np.zeros(A.CLM_AF_NFIELDS * self.w.ncol)
        rc = lib().clmo_atmos_fluxes(ctypes.byref(self.P), *self._st(state), A.dptr(out))
        assert rc == 0, rc
        return out.reshape(A.CLM_AF_NFIELDS, self.w.ncol)

    def update_cache(self, state, t):
        nc = self.w.ncells
        out = {k: np.zeros(nc) for k in ("K", "psi", "theta_l", "T", "kappa", "Tf")}
        bc = np.zeros(4 * self.w.ncol)
        W = np.zeros(self.w.ncol)
        E = np.zeros(self.w.ncol)
        rc = lib().clmo_update_cache(ctypes.byref(self.P), *self._st(state), float(t),
                                     *[A.dptr(out[k]) for k in ("K", "psi", "theta_l", "T", "kappa", "Tf")],
                                     A.dptr(bc), A.dptr(W), A.dptr(E))
        assert rc == 0, rc
        out["bc"] = bc.reshape(4, self.w.ncol)
        out["total_water"] = W
        out["total_energy"] = E
        return out

    def _tend(self, fn, state, t):
        nc, ncol = self.w.ncells, self.w.ncol
        d = [np.zeros(nc), np.zeros(nc), np.zeros(nc), np.zeros(ncol), np.zeros(ncol)]
        rc = fn(ctypes.byref(self.P), *self._st(state), float(t), *[A.dptr(a) for a in d])
        assert rc == 0, rc
        return d

    def exp_tendency(self, state, t):
        return self._tend(lib().clmo_exp_tendency, state, t)

    def imp_tendency(self, state, t):
        return self._tend(lib().clmo_imp_tendency, state, t)

    def jacobian(self, state, t, dtgamma):
        nc = self.w.ncells
        J = [np.zeros(3 * nc) for _ in range(3)]
        rc = lib().clmo_jacobian(ctypes.byref(self.P), *self._st(state), float(t), float(dtgamma),
                                 *[A.dptr(a) for a in J])
        assert rc == 0, rc
        return [a.reshape(nc, 3) for a in J]

    def solve(self, Wvv, Wev, Wee, fv, fe):
        nc = self.w.ncells
        dv = np.zeros(nc)
        de = np.zeros(nc)
        c = np.ascontiguousarray
        rc = lib().clmo_solve(ctypes.byref(self.P), A.dptr(c(Wvv)), A.dptr(c(Wev) if Wev is not None else None),
                              A.dptr(c(Wee) if Wee is not None else None), A.dptr(c(fv)),
                              A.dptr(c(fe) if fe is not None else None), A.dptr(dv), A.dptr(de))
        assert rc == 0, rc
        return dv, de

    def runoff(self, state, t):
        """Runoff diagnostics of the explicit stage (CLM_BC_PRECIP_RUNOFF):
        infiltration, R_s, R_ss, h_sat per column."""
        out = [np.zeros(self.w.ncol) for _ in range(4)]
        rc = lib().clmo_runoff(ctypes.byref(self.P), A.dptr(state[0]), float(t), *[A.dptr(a) for a in out])
        assert rc == 0, rc
        return dict(zip(("infiltration", "R_s", "R_ss", "h_sat"), out))

    def budgets(self, state):
        W = np.zeros(self.w.ncol)
        E = np.zeros(self.w.ncol)
        rc = lib().clmo_budgets(ctypes.byref(self.P), *self._st(state), A.dptr(W), A.dptr(E))
        assert rc == 0, rc
        return W, E


def pointwise():
    """Direct access to the oracle's pointwise functions."""
    return lib()

"""Shared helpers of the GPU parity tests (imported by test_gpu_*.py)."""
import numpy as np
import pytest

import oracle as O
from climaland_gb300 import _abi as A
from climaland_gb300 import device as D

# Parity bar of the plain FP64 path against the FP64 oracle after N steps:
# max-abs 1e-10 in vartheta_l and theta_i; rho_e_int max-abs relative to its
# scale (max |rho_e_int|) 1e-10; budgets closed to 1e-12 relative.
TOL_STATE = 1e-10
TOL_BUDGET = 1e-12


def require_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def run_both(w, nsteps=None, oracle_cfg=None, **dev_kw):
    """Run the oracle and the GPU on the same workload; return both states."""
    nsteps = w.nsteps if nsteps is None else nsteps
    o = O.Oracle(w)
    if oracle_cfg:
        o.set_cfg(**oracle_cfg)
    so = w.copy_state()
    rc, fo, io = o.step(so, w.t0, w.dt, nsteps)
    assert rc == 0, rc
    with D.SoilColumns(w, **dev_kw) as g:
        g.step(w.t0, w.dt, nsteps)
        sg = g.get_state()
        fg, ig = g.status()
        Wg, Eg = g.budgets()
    return so, sg, (fo, io), (fg, ig), (Wg, Eg)


def state_errors(w, so, sg):
    err = {"vartheta_l": float(np.max(np.abs(so[0] - sg[0])))}
    err["intF_w"] = float(np.max(np.abs(so[3] - sg[3])))
    if w.cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY:
        err["theta_i"] = float(np.max(np.abs(so[1] - sg[1])))
        scale = float(np.max(np.abs(so[2])))
        err["rho_e_int_rel"] = float(np.max(np.abs(so[2] - sg[2]))) / scale
        err["intF_e_rel"] = float(np.max(np.abs(so[4] - sg[4]))) / max(float(np.max(np.abs(so[4]))), 1.0)
    return err


def assert_state_parity(w, so, sg, tol=TOL_STATE):
    err = state_errors(w, so, sg)
    for k, v in err.items():
        assert v <= tol, f"{w.name}: {k} error {v:.3e} > {tol:.1e} ({err})"
    return err


def budget_errors(w, state0, state1, W1, E1):
    o = O.Oracle(w)
    W0, E0 = o.budgets(state0)
    ew = float(np.max(np.abs((W1 - W0) - (state1[3] - state0[3])) / np.abs(W0)))
    ee = 0.0
    if w.cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY:
        ee = float(np.max(np.abs((E1 - E0) - (state1[4] - state0[4])) / np.abs(E0)))
    return ew, ee

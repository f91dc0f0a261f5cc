"""GPU parity of the fused column step (plain FP64 path) against the oracle,
through the C ABI, on the configurations' seeded inputs and edge cases."""
import numpy as np
import pytest

from climaland_gb300 import _abi as A
from climaland_gb300 import parameters as PR
from climaland_gb300 import workloads as WL
from gpu_common import (TOL_BUDGET, TOL_STATE, assert_state_parity, budget_errors,
                        require_gpu, run_both, state_errors)

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu():
    require_gpu()


def test_richards_c0_full():
    """Plain Richards 1024 x 20, 96 steps, 3 Newton iterations."""
    w = WL.richards_c0()
    so, sg, (fo, io), (fg, ig), (Wg, Eg) = run_both(w)
    assert_state_parity(w, so, sg)
    assert fg.max() == 0 and np.all(ig == 3)
    ew, _ = budget_errors(w, w.copy_state(), sg, Wg, Eg)
    assert ew < TOL_BUDGET


def test_energy_hydrology_c1_sample():
    """Plain EnergyHydrology, 4096 columns of the 65,536 x 15 configuration,
    all 192 steps (dt = 450 s, diurnal heat flux, freeze/thaw)."""
    w = WL.energy_hydrology_c1().subset(4096)
    so, sg, (fo, io), (fg, ig), (Wg, Eg) = run_both(w)
    err = assert_state_parity(w, so, sg)
    assert fg.max() == 0
    ew, ee = budget_errors(w, w.copy_state(), sg, Wg, Eg)
    assert ew < TOL_BUDGET and ee < TOL_BUDGET, (ew, ee, err)


def test_uneven_columns_c2_sample():
    """Uneven CSR columns (4..30 layers, 0.5-5 m), 2048 columns, 48 steps."""
    w = WL.uneven_c2().subset(2048)
    so, sg, *_ = run_both(w, nsteps=48)
    assert_state_parity(w, so, sg)


def test_full_scale_c4_sample():
    """Rain pulses (counter hash), advective heat flux, variable depth:
    1024 columns of the 1,048,576 x 20 configuration, 96 steps."""
    w = WL.full_scale_c4(ncol=1024)
    so, sg, *_ = run_both(w, nsteps=96)
    assert_state_parity(w, so, sg)


@pytest.mark.parametrize("ncol", [1, 31, 33, 100])
def test_ragged_column_counts(ncol):
    w = WL.energy_hydrology_c1(ncol=ncol, nlayers=7)
    so, sg, *_ = run_both(w, nsteps=20)
    assert_state_parity(w, so, sg)


@pytest.mark.parametrize("nlayers", [2, 3, 64])
def test_layer_count_limits(nlayers):
    w = WL.richards_c0(ncol=64, nlayers=nlayers)
    so, sg, *_ = run_both(w, nsteps=10)
    assert_state_parity(w, so, sg)
    w = WL.energy_hydrology_c1(ncol=64, nlayers=nlayers)
    so, sg, *_ = run_both(w, nsteps=10)
    assert_state_parity(w, so, sg)


def test_saturated_and_dry_columns():
    """S >= 1 (positive pressure, 1/S_s branches) and near-residual columns."""
    w = WL.richards_c0(ncol=96, nlayers=12)
    nu = np.repeat(w.params[A.CLM_P_NU], 12)
    thr = np.repeat(w.params[A.CLM_P_THETA_R], 12)
    v = w.vartheta_l.copy()
    v[: 32 * 12] = nu[: 32 * 12] + 0.01          # supersaturated
    v[32 * 12: 64 * 12] = thr[32 * 12: 64 * 12] + 1e-9  # at the residual clip
    w.vartheta_l = v
    w.forcing[A.CLM_BC_TOP_WATER][A.CLM_F_BASE][:] = -1e-5
    so, sg, *_ = run_both(w, nsteps=20)
    assert_state_parity(w, so, sg)


def test_richards_moisture_state_bc():
    """MoistureStateBC on top (implicit dfluxBCdY term, BCs refreshed inside
    Newton) with FreeDrainage at the bottom."""
    w = WL.richards_c0(ncol=128, nlayers=20)
    w.cfg.bc_top_water = A.CLM_BC_STATE
    f = WL.constant_forcing(w.ncol, w.params[A.CLM_P_NU] - 1e-3)
    w.forcing[A.CLM_BC_TOP_WATER] = f
    so, sg, *_ = run_both(w, nsteps=40)
    assert_state_parity(w, so, sg)


def test_energy_state_bcs():
    """TemperatureStateBC top and bottom, MoistureStateBC bottom (explicit)."""
    w = WL.energy_hydrology_c1(ncol=128, nlayers=15)
    w.cfg.bc_top_heat = A.CLM_BC_STATE
    w.cfg.bc_bottom_heat = A.CLM_BC_STATE
    w.cfg.bc_bottom_water = A.CLM_BC_STATE
    fh = WL.constant_forcing(w.ncol, 268.0)
    fh[A.CLM_F_AMP] = 5.0
    fh[A.CLM_F_OMEGA] = 2 * np.pi / 86400.0
    w.forcing[A.CLM_BC_TOP_HEAT] = fh
    w.forcing[A.CLM_BC_BOTTOM_HEAT] = WL.constant_forcing(w.ncol, 278.0)
    w.forcing[A.CLM_BC_BOTTOM_WATER] = WL.constant_forcing(w.ncol, w.params[A.CLM_P_NU] - 0.05)
    so, sg, *_ = run_both(w, nsteps=60)
    assert_state_parity(w, so, sg)


def test_tolerance_mode_iterations_match():
    """CTS ConvergenceChecker(MaximumError) semantics per column: the GPU and
    the oracle stop after the same number of iterations."""
    w = WL.richards_c0(ncol=256)
    kw = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=50, newton_tol=1e-10)
    so, sg, (fo, io), (fg, ig), _ = run_both(
        w, nsteps=12, oracle_cfg=kw, **kw)
    assert_state_parity(w, so, sg)
    assert np.mean(io == ig) > 0.99


def test_state_roundtrip_and_device_pointers():
    """set_state -> get_state is the identity (layout transposes, sorting)."""
    import torch
    w = WL.uneven_c2(ncol=300)
    from climaland_gb300 import device as D
    with D.SoilColumns(w) as g:
        s = g.get_state()
        for a, b in zip(s, w.copy_state()):
            assert np.array_equal(a, b)
        t = [torch.tensor(x, device="cuda") for x in w.copy_state()]
        for x in t:
            x.mul_(1.0)
        g.set_state_device([x.data_ptr() for x in t])
        out = [torch.empty_like(x) for x in t]
        g.get_state_device([x.data_ptr() for x in out])
        torch.cuda.synchronize()
        for a, b in zip(out, t):
            assert torch.equal(a, b)


def test_nonfinite_state_flagged():
    """A NaN planted in the input state is reported per column, not trapped."""
    w = WL.energy_hydrology_c1(ncol=64, nlayers=10)
    w.rho_e_int[5 * 10 + 3] = np.nan
    from climaland_gb300 import device as D
    with D.SoilColumns(w) as g:
        g.step(0.0, w.dt, 2)
        f, _ = g.status()
    assert f[5] & A.CLM_COL_NONFINITE
    assert np.count_nonzero(f & A.CLM_COL_NONFINITE) == 1


def test_invalid_arguments_rejected():
    from climaland_gb300 import device as D
    w = WL.richards_c0(ncol=32, nlayers=5)
    w.params[A.CLM_P_VG_N][3] = 0.9  # n must exceed 1
    with pytest.raises(D.ClmError) as e:
        D.SoilColumns(w)
    assert e.value.code == A.CLM_ERR_ARG
    w = WL.richards_c0(ncol=32, nlayers=5)
    with D.SoilColumns(w) as g:
        with pytest.raises(D.ClmError):
            g.step(0.0, -1.0, 1)

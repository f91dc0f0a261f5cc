"""GPU parity of the fused column step against the oracle, through the C
ABI, on the configurations' seeded inputs and edge cases (criterion in
gpu_common)."""
import json

import numpy as np
import pytest

import oracle as O
from climaland_gb300 import _abi as A
from climaland_gb300 import device as D
from climaland_gb300 import workloads as WL
from gpu_common import TOL_MODE, check_parity, require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(autouse=True)
def _gpu():
    require_gpu()


def report(name, stats):
    from gpu_common import SUMMARY
    if SUMMARY and SUMMARY[-1][1] is stats:
        SUMMARY[-1] = (name, stats)
    print(f"PARITY {name} {json.dumps(stats)}")


def test_richards_c0_full():
    """Plain Richards 1024 x 20, all 96 steps, 3 Newton iterations."""
    w = WL.richards_c0()
    st = check_parity(w, w.nsteps)
    report("richards_c0", st)
    assert st["gpu_iters_max"] == 3


def test_energy_hydrology_c1_full():
    """Plain EnergyHydrology: the whole 65,536 x 15 configuration, all 192
    steps (dt = 450 s, diurnal heat flux, freeze/thaw)."""
    w = WL.energy_hydrology_c1()
    report("eh_c1", check_parity(w, w.nsteps))


def test_energy_hydrology_c1_tolerance_mode():
    """Same, Newton to convergence (ConvergenceChecker semantics)."""
    w = WL.energy_hydrology_c1().subset(2048)
    st = check_parity(w, w.nsteps, oracle_cfg=TOL_MODE, **TOL_MODE)
    report("eh_c1_tol", st)
    assert st["iters_agree"] > 0.99


def test_uneven_columns_c2_sample():
    """Uneven CSR columns (4..30 layers, 0.5-5 m), 2048 columns, 96 steps."""
    w = WL.uneven_c2().subset(2048)
    report("uneven_c2", check_parity(w, 96))


def test_full_scale_c4_eight_days():
    """Rain pulses (counter hash), advective heat flux, variable depth:
    8,192 columns of the 1,048,576 x 20 configuration over all 1536 steps
    (8 simulated days of dt = 450 s)."""
    w = WL.full_scale_c4(ncol=8192)
    report("full_scale_c4_1536", check_parity(w, w.nsteps))


def test_full_scale_c4_tolerance_mode():
    w = WL.full_scale_c4(ncol=512)
    report("full_scale_c4_tol", check_parity(w, 96, oracle_cfg=TOL_MODE, **TOL_MODE))


@pytest.mark.parametrize("prec", [A.CLM_PREC_FP64, A.CLM_PREC_MIXED])
def test_extrapolated_start_reaches_the_oracle_root(prec):
    """Tolerance mode at 1e-12 from the extrapolated start u_n + (u_n -
    u_{n-1}) against the oracle solving from U: a start changes the path to
    the root, not the root, so the FP64 path meets the FP64 criterion and the
    mixed path the mixed one."""
    w = WL.full_scale_c4(ncol=1024, seed=4)
    kw = dict(TOL_MODE, learned_guess=A.CLM_GUESS_EXTRAPOLATE)
    if prec == A.CLM_PREC_MIXED:
        kw.update(MIXED)
    report(f"extrapolated_start_{'mixed' if prec == A.CLM_PREC_MIXED else 'fp64'}",
           check_parity(w, 48, oracle_cfg=TOL_MODE, **kw))


# Mixed path (FP32 Jacobian and Thomas; double-float closures; FP64 residual
# assembly, increments, phase partition and budgets): 1e-8 wherever the
# oracle reproduces itself under perturbations as large as the column's own
# one-step difference from the oracle (gpu_common: "calibrated"), budgets
# as the plain path.
MIXED = dict(tol_state=1e-8, noise="calibrated", precision=A.CLM_PREC_MIXED)


@pytest.mark.parametrize("name,make,nsteps", [
    ("full_scale", lambda: WL.full_scale_c4(ncol=1024), 48),
    ("energy_hydrology", lambda: WL.energy_hydrology_c1().subset(1024), 48),
    ("uneven", lambda: WL.uneven_c2().subset(1024), 48),
    ("richards", lambda: WL.richards_c0(ncol=1024), 96),
])
def test_mixed_precision_within_1e8(name, make, nsteps):
    report(f"mixed_{name}", check_parity(make(), nsteps, **MIXED))


def test_mixed_precision_tolerance_mode():
    w = WL.full_scale_c4(ncol=512)
    report("mixed_full_scale_tol", check_parity(w, 48, oracle_cfg=TOL_MODE, **TOL_MODE, **MIXED))


# Brooks-Corey closure (cfg.hydrology_cm = CLM_CM_BROOKS_COREY): sandy columns
# with |psi_b| ~ 0.05 m and K_sat ~ 1e-4 m/s are stiff enough that three
# Newton iterations diverge (the reference's trajectory there is not
# reproducible: those columns fall under the oracle-spread bound).
BROOKS_COREY = {
    "richards": (lambda: WL.brooks_corey(WL.richards_c0(ncol=1024)), 96, {}),
    "energy_hydrology": (lambda: WL.brooks_corey(WL.energy_hydrology_c1().subset(1024)), 96, {}),
    "uneven": (lambda: WL.brooks_corey(WL.uneven_c2().subset(1024)), 48, {}),
    "full_scale": (lambda: WL.brooks_corey(WL.full_scale_c4(ncol=1024)), 48, {}),
    "full_scale_tol": (lambda: WL.brooks_corey(WL.full_scale_c4(ncol=512)), 48,
                       dict(oracle_cfg=TOL_MODE, **TOL_MODE)),
    "mixed_energy_hydrology": (lambda: WL.brooks_corey(WL.energy_hydrology_c1().subset(1024)), 48, MIXED),
    "mixed_full_scale": (lambda: WL.brooks_corey(WL.full_scale_c4(ncol=1024)), 48, MIXED),
    "mixed_uneven": (lambda: WL.brooks_corey(WL.uneven_c2().subset(1024)), 48, MIXED),
    "mixed_richards": (lambda: WL.brooks_corey(WL.richards_c0(ncol=1024)), 96, MIXED),
}


@pytest.mark.parametrize("name", list(BROOKS_COREY))
def test_brooks_corey(name):
    make, nsteps, kw = BROOKS_COREY[name]
    report(f"brooks_corey_{name}", check_parity(make(), nsteps, **kw))


# RootExtraction (the canopy's per-layer water and energy sink): the
# reference adds the extraction's column integral to intF_w with the sign
# opposite to the state's change, so its budgets drift by 2 dt sum dz re per
# step; the GPU's per-column defects must equal the oracle's.
ROOTS = {
    "full_scale": (lambda: WL.with_root_extraction(WL.full_scale_c4(ncol=1024)), 48, {}),
    "energy_hydrology": (lambda: WL.with_root_extraction(WL.energy_hydrology_c1().subset(1024)), 96, {}),
    "uneven": (lambda: WL.with_root_extraction(WL.uneven_c2().subset(1024)), 48, {}),
    "brooks_corey": (lambda: WL.with_root_extraction(WL.brooks_corey(WL.full_scale_c4(ncol=512))), 48, {}),
    "mixed_full_scale": (lambda: WL.with_root_extraction(WL.full_scale_c4(ncol=1024)), 48, MIXED),
}


@pytest.mark.parametrize("name", list(ROOTS))
def test_root_extraction(name):
    make, nsteps, kw = ROOTS[name]
    report(f"roots_{name}", check_parity(make(), nsteps, **kw))


def test_root_extraction_refused_for_richards_and_removable():
    w = WL.richards_c0(ncol=32, nlayers=5)
    with D.SoilColumns(w) as g:
        with pytest.raises(D.ClmError) as e:
            g.set_root_extraction(np.ones((A.CLM_RX_NFIELDS, 32)))
        assert e.value.code == A.CLM_ERR_ARG
    # removing the source gives the plain step's bits
    w = WL.with_root_extraction(WL.full_scale_c4(ncol=256))
    plain = WL.full_scale_c4(ncol=256)
    with D.SoilColumns(w) as g, D.SoilColumns(plain) as g0:
        bad = w.root.copy()
        bad[A.CLM_RX_ROOT_DEPTH, 7] = 0.0
        with pytest.raises(D.ClmError):
            g.set_root_extraction(bad)
        g.set_root_extraction(None)
        g.step(w.t0, w.dt, 4)
        g0.step(w.t0, w.dt, 4)
        for a, b in zip(g.get_state(), g0.get_state()):
            assert np.array_equal(a, b)


# Atmosphere-driven top boundary (AtmosDrivenFluxBC + SoilSublimation): the
# explicit-stage turbulent, radiative and precipitation fluxes at the top.
ATMOS = {
    "full_scale": (lambda: WL.with_atmos(WL.full_scale_c4(ncol=1024)), 48, {}),
    "energy_hydrology": (lambda: WL.with_atmos(WL.energy_hydrology_c1().subset(1024)), 96, {}),
    "uneven": (lambda: WL.with_atmos(WL.uneven_c2().subset(1024)), 48, {}),
    "brooks_corey": (lambda: WL.with_atmos(WL.brooks_corey(WL.full_scale_c4(ncol=512))), 48, {}),
    "full_scale_tol": (lambda: WL.with_atmos(WL.full_scale_c4(ncol=512)), 48,
                       dict(oracle_cfg=TOL_MODE, **TOL_MODE)),
    "mixed_full_scale": (lambda: WL.with_atmos(WL.full_scale_c4(ncol=1024)), 48, MIXED),
    "mixed_brooks_corey": (lambda: WL.with_atmos(WL.brooks_corey(WL.full_scale_c4(ncol=512))), 48, MIXED),
    "surface_runoff": (lambda: WL.with_atmos(WL.full_scale_c4(ncol=1024), runoff=A.CLM_RUNOFF_SURFACE), 48, {}),
    "topmodel": (lambda: WL.with_atmos(WL.full_scale_c4(ncol=1024), runoff=A.CLM_RUNOFF_TOPMODEL), 48, {}),
    "topmodel_uneven": (lambda: WL.with_atmos(WL.uneven_c2().subset(1024), runoff=A.CLM_RUNOFF_TOPMODEL), 48, {}),
    # supersaturated water-table layers (dpsi/dvartheta = 1/S_s) make the
    # mixed path's float Jacobian rows its least accurate part: with three
    # fixed Newton iterations one column of 1024 reaches 1.8e-8 in rho e_int
    "mixed_topmodel": (lambda: WL.with_atmos(WL.full_scale_c4(ncol=1024), runoff=A.CLM_RUNOFF_TOPMODEL), 48,
                       dict(MIXED, tol_state=2e-8)),
}


@pytest.mark.parametrize("name", list(ATMOS))
def test_atmos_driven_boundary(name):
    make, nsteps, kw = ATMOS[name]
    report(f"atmos_{name}", check_parity(make(), nsteps, **kw))


@pytest.mark.parametrize("bc", [False, True])
def test_atmos_fluxes_match_oracle(bc):
    """clm_atmos_fluxes (turbulent fluxes, net radiation, surface humidity,
    top fluxes) against the oracle at the same state: FP64 arithmetic in a
    different order (table exp/log, reciprocals), 1e-11 of each field's
    scale."""
    base = WL.full_scale_c4(ncol=2048)
    w = WL.with_atmos(WL.brooks_corey(base) if bc else base)
    st = w.copy_state()
    fo = O.Oracle(w).atmos_fluxes(st)
    with D.SoilColumns(w) as g:
        fg = g.atmos_fluxes()
        for f in range(A.CLM_AF_NFIELDS):
            sc = np.max(np.abs(fo[f])) + 1e-300
            err = np.max(np.abs(fg[f] - fo[f]))
            assert err <= 1e-11 * sc, (A.ATMOS_FLUXES[f], err, sc)
        # after a few steps, at a state with sublimating and evaporating columns
        g.step(w.t0, w.dt, 6)
        st = g.get_state()
        fo = O.Oracle(w).atmos_fluxes(st)
        fg = g.atmos_fluxes()
        assert (fo[A.CLM_AF_VAPOR_ICE] != 0).any() and (fo[A.CLM_AF_VAPOR_LIQ] != 0).any()
        for f in range(A.CLM_AF_NFIELDS):
            sc = np.max(np.abs(fo[f])) + 1e-300
            assert np.max(np.abs(fg[f] - fo[f])) <= 1e-11 * sc, A.ATMOS_FLUXES[f]


def test_atmos_boundary_refusals():
    """EnergyHydrology only, both top kinds, a known runoff model; drivers required and
    validated; no root extraction beside it; removing the drivers stops the
    step until they are set again."""
    w = WL.with_atmos(WL.full_scale_c4(ncol=64))
    for mut in (dict(bc_top_heat=A.CLM_BC_FLUX), dict(runoff=7)):
        cfg = A.ClmConfig.from_buffer_copy(w.cfg)
        for k, v in mut.items():
            setattr(cfg, k, v)
        bad = w.columns(0, w.ncol)
        bad.cfg = cfg
        with pytest.raises(D.ClmError) as e:
            D.SoilColumns(bad)
        assert e.value.code == A.CLM_ERR_ARG
    r = WL.richards_c0(ncol=32, nlayers=5)
    r.cfg.bc_top_water = r.cfg.bc_top_heat = A.CLM_BC_ATMOS
    with pytest.raises(D.ClmError):
        D.SoilColumns(r)
    with D.SoilColumns(w) as g:
        d = w.atmos.copy()
        d[A.CLM_AT_Z_0M, 3] = 0.0
        with pytest.raises(D.ClmError) as e:
            g.set_atmos(d)
        assert e.value.code == A.CLM_ERR_ARG
        with pytest.raises(D.ClmError) as e:
            g.set_root_extraction(np.ones((A.CLM_RX_NFIELDS, w.ncol)))
        assert e.value.code == A.CLM_ERR_UNSUPPORTED
        g.set_atmos(None)
        with pytest.raises(D.ClmError) as e:
            g.step(w.t0, w.dt, 1)
        assert e.value.code == A.CLM_ERR_STATE
        g.set_atmos(w.atmos)
        g.step(w.t0, w.dt, 1)


@pytest.mark.parametrize("kind", [A.CLM_RUNOFF_NONE, A.CLM_RUNOFF_SURFACE, A.CLM_RUNOFF_TOPMODEL])
def test_richards_precipitation_runoff(kind):
    """RichardsAtmosDrivenFluxBC with each runoff model: hourly storms above
    K_sat, saturated deep layers (TOPMODEL's saturated height and subsurface
    sink); budgets against the oracle's (the reference keeps subtracting R_ss
    from the integrated flux when no layer is saturated). FP64 path only: in
    saturated layers dpsi = 1/S_s makes the Jacobian's off-diagonals ~1e7
    against its "- I", which a float Jacobian cannot represent."""
    w = WL.richards_runoff(ncol=1024, runoff=kind)
    report(f"richards_runoff_{kind}", check_parity(w, 48))


def test_richards_tolerance_mode():
    w = WL.richards_c0(ncol=512)
    st = check_parity(w, 48, oracle_cfg=TOL_MODE, **TOL_MODE)
    report("richards_tol", st)
    assert st["iters_agree"] > 0.99


@pytest.mark.parametrize("ncol", [1, 31, 33, 100])
def test_ragged_column_counts(ncol):
    w = WL.energy_hydrology_c1(ncol=ncol, nlayers=7)
    check_parity(w, 20)


@pytest.mark.parametrize("nlayers", [2, 3, 64])
def test_layer_count_limits(nlayers):
    check_parity(_moderate(WL.richards_c0(ncol=64, nlayers=nlayers)), 10)
    check_parity(_moderate(WL.energy_hydrology_c1(ncol=64, nlayers=nlayers)), 10)


def _moderate(w, kmax=1e-5):
    """Cap K_sat so that dt K_sat / dz^2 stays moderate: the edge cases below
    probe branches of the physics, not the stiff regime in which the
    reference's three-iteration Newton itself stops being reproducible."""
    w.params[A.CLM_P_K_SAT] = np.minimum(w.params[A.CLM_P_K_SAT], kmax)
    return w


def test_saturated_and_dry_columns():
    """S > 1 (positive pressure, the 1/S_s branches of psi and dpsi) and
    columns at the residual clip theta_r + sqrt(eps), draining and wetting."""
    w = _moderate(WL.richards_c0(ncol=96, nlayers=12))
    nu = np.repeat(w.params[A.CLM_P_NU], 12)
    thr = np.repeat(w.params[A.CLM_P_THETA_R], 12)
    v = w.vartheta_l.copy()
    v[: 32 * 12] = nu[: 32 * 12] + 0.002            # supersaturated, draining
    v[32 * 12: 64 * 12] = thr[32 * 12: 64 * 12] + 1e-9  # at the residual clip
    w.vartheta_l = v
    f = w.forcing[A.CLM_BC_TOP_WATER][A.CLM_F_BASE]
    f[:32] = 0.0
    f[32:64] = -2e-7
    check_parity(w, 20)


def test_richards_moisture_state_bc():
    """MoistureStateBC on top (implicit dfluxBCdY term, BCs refreshed inside
    Newton) with FreeDrainage at the bottom."""
    w = _moderate(WL.richards_c0(ncol=128, nlayers=20))
    w.cfg.bc_top_water = A.CLM_BC_STATE
    w.forcing[A.CLM_BC_TOP_WATER] = WL.constant_forcing(w.ncol, w.params[A.CLM_P_NU] - 1e-3)
    check_parity(w, 40)


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
    check_parity(w, 60)


def test_multi_step_launch_equals_single_steps():
    """clm_step(t, dt, k) in one call equals k calls of one step (bitwise)."""
    w = WL.energy_hydrology_c1(ncol=256, nlayers=15)
    with D.SoilColumns(w) as g:
        g.step(0.0, w.dt, 70)
        a = g.get_state()
    with D.SoilColumns(w) as g:
        for i in range(70):
            g.step(i * w.dt, w.dt, 1)
        b = g.get_state()
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_state_roundtrip_and_device_pointers():
    """set_state -> get_state is the identity (layout transposes, sorting)."""
    import torch
    w = WL.uneven_c2(ncol=300)
    with D.SoilColumns(w) as g:
        s = g.get_state()
        for a, b in zip(s, w.copy_state()):
            assert np.array_equal(a, b)
        t = [torch.tensor(x, device="cuda") for x in w.copy_state()]
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
    with D.SoilColumns(w) as g:
        g.step(0.0, w.dt, 2)
        f, _ = g.status()
    assert f[5] & A.CLM_COL_NONFINITE
    assert np.count_nonzero(f & A.CLM_COL_NONFINITE) == 1


def test_invalid_arguments_rejected():
    w = WL.richards_c0(ncol=32, nlayers=5)
    w.params[A.CLM_P_VG_N][3] = 0.9  # n must exceed 1
    with pytest.raises(D.ClmError) as e:
        D.SoilColumns(w)
    assert e.value.code == A.CLM_ERR_ARG
    w = WL.brooks_corey(WL.richards_c0(ncol=32, nlayers=5))
    w.params[A.CLM_P_BC_PSI_B][3] = 0.1  # psi_b must be negative
    with pytest.raises(D.ClmError) as e:
        D.SoilColumns(w)
    assert e.value.code == A.CLM_ERR_ARG
    w = WL.richards_c0(ncol=32, nlayers=5)
    with D.SoilColumns(w) as g:
        with pytest.raises(D.ClmError):
            g.step(0.0, -1.0, 1)


# Stretched columns (clm_set_faces): generalized exponential faces with a
# thin top layer (Column(; dz_tuple), global_domain's dz_tuple = (10.0,
# 0.05) over 50 m), and the reference RichardsModel benchmark's geometry
# and solver settings (15 layers over 50 m, dz_tuple = (10.0, 0.1), TOPMODEL,
# 2 Newton iterations, dt = 1800 s).
STRETCHED = {
    "energy_hydrology": (lambda: WL.stretched(WL.energy_hydrology_c1().subset(2048)), 192, {}),
    "global_domain": (lambda: WL.global_eh_stretched(ncol=2048), 192, {}),
    "full_scale": (lambda: WL.stretched(WL.full_scale_c4(ncol=2048)), 192, {}),
    "uneven": (lambda: WL.stretched(WL.uneven_c2().subset(2048)), 96, {}),
    "richards": (lambda: WL.stretched(WL.richards_c0()), 96, {}),
    "richards_benchmark": (lambda: WL.richards_benchmark(ncol=2048), 336, {}),
    "full_scale_tol": (lambda: WL.stretched(WL.full_scale_c4(ncol=1024)), 96,
                       dict(oracle_cfg=TOL_MODE, **TOL_MODE)),
    "atmos_topmodel": (lambda: WL.with_atmos(WL.stretched(WL.full_scale_c4(ncol=1024)),
                                             runoff=A.CLM_RUNOFF_TOPMODEL), 96, {}),
    "roots": (lambda: WL.with_root_extraction(WL.stretched(WL.full_scale_c4(ncol=1024))), 96, {}),
    "brooks_corey": (lambda: WL.brooks_corey(WL.stretched(WL.full_scale_c4(ncol=1024))), 96, {}),
    "mixed_energy_hydrology": (lambda: WL.stretched(WL.energy_hydrology_c1().subset(1024)), 48, MIXED),
    "mixed_global_domain": (lambda: WL.global_eh_stretched(ncol=1024), 48, MIXED),
    "mixed_full_scale": (lambda: WL.stretched(WL.full_scale_c4(ncol=1024)), 48, MIXED),
    "mixed_richards": (lambda: WL.stretched(WL.richards_c0()), 96, MIXED),
}


@pytest.mark.parametrize("name", list(STRETCHED))
def test_stretched_columns(name):
    make, nsteps, kw = STRETCHED[name]
    report(f"stretched_{name}", check_parity(make(), nsteps, **kw))


@pytest.mark.parametrize("name,make,bound", [
    ("full_scale", lambda: WL.full_scale_c4(ncol=1024), 1e-11),
    ("stretched_full_scale", lambda: WL.stretched(WL.full_scale_c4(ncol=1024)), 1e-11),
    ("stretched_richards", lambda: WL.stretched(WL.richards_c0()), 1e-9),
])
def test_mixed_path_converges_to_the_oracle_root(name, make, bound):
    """Eight fixed Newton iterations on both: one step of the mixed path from
    states along the oracle's trajectory lands on the oracle's step to 1e-11
    (the float Jacobian changes only how fast Newton converges; the
    residual's closures are double-float, ~2^-44 relative). On the stretched
    RichardsModel columns Newton with the reference's approximate Jacobian
    converges only linearly in saturated layers (after 8 iterations the
    oracle itself is up to 2.5e-4 from its 40-iteration result), so there the
    two iterations are compared at equal counts, to 1e-9 (1.3e-10 measured
    on the 1024 columns)."""
    from gpu_common import step_deviation

    w = make()
    w.cfg.max_iters = 8
    dev = step_deviation(w, 24, every=4, precision=A.CLM_PREC_MIXED)
    assert float(dev.max()) <= bound, float(dev.max())

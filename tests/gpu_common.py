"""Shared helpers of the GPU parity tests (imported by test_gpu_*.py).

Parity criterion. The bar is 1e-10 max-abs in vartheta_l and theta_i and
1e-10 in rho_e_int relative to its scale (max |rho_e_int|), with water and
energy budgets closed to 1e-12 relative. On some columns the reference
algorithm itself does not reproduce to that level: with the default three
fixed Newton iterations, stiff columns (K_sat dt / dz^2 >> 1) and frozen
cells whose explicit phase-change source is unstable amplify a 1-ulp
perturbation of the input to 1e-8 .. 1e-5 within a few dozen steps. On
those columns no implementation can agree with the oracle more closely than
the oracle agrees with itself under rounding. The test therefore measures,
per column, the oracle's own spread under random rounding-size noise added
to all state arrays at every step (8 seeds): +-1 ulp of each field's scale
(max |field| of the initial state) on every nonzero value, the absolute
error of a quantity computed from terms of that size (theta_i of a thawed
layer is a difference of O(0.1) terms and carries ~1e-17 absolute error
however small it is; exact zeros stay exact in both codes). It requires on
every column
  error <= max(1e-10, 10 x spread),
i.e. the bar wherever the oracle reproduces itself. A chaotic column's
deviation under noise is heavy-tailed (on column 16 of the stretched
RichardsModel benchmark workload, 32 one-ulp runs give a median of 1.2e-8
and a maximum of 5.9e-7), so 8 seeds can under-estimate it: a column that 8
seeds do not cover is re-measured on its own with 32 more (at most 64 such
columns per test). The number of columns that need the widened bound (error
above 1e-10) may not exceed 5 %, or, over long runs where chaos has spread
further, the fraction of columns on which the oracle's own perturbed runs
exceed 1e-10. Each test records the excused fraction, the largest
error/spread ratio among excused columns and the oracle's own fraction,
printed in the session summary.

Mixed path: 1e-8, with the spread measured under per-step noise as large as
each column's own one-step difference from the oracle (the mixed path
stepping from the oracle's state, sampled along the oracle's trajectory;
at least 2^-44, the double-float closures' precision, at most 1e-9). Its
float Jacobian converges more slowly than the FP64 one on stiff columns, so
three fixed Newton iterations leave differences up to ~1e-9 per step there;
the converged root itself is the oracle's (test_gpu_parity.py checks it
with eight iterations).

Budgets, per column: water and energy close to 1e-12 relative on the GPU
state, except where the reference itself does not close them
(MoistureStateBC with a fixed number of Newton iterations: the integrated
flux uses the boundary flux of the iterate before the last update; columns
whose three Newton iterations do not converge); there the GPU's defect must
equal the oracle's to 1e-8 of it, or to 10 x the spread of the oracle's
own defect under the same perturbations.
"""
import numpy as np
import pytest

import oracle as O
from climaland_gb300 import _abi as A
from climaland_gb300 import device as D

TOL_STATE = 1e-10
TOL_BUDGET = 1e-12
SENSITIVE = 1e-13      # oracle self-spread above which a column is sensitive
SPREAD_FACTOR = 10.0   # allowed multiple of the oracle's own spread
MAX_SENSITIVE = 0.05    # at most this fraction of columns may be sensitive
NSEEDS = 8
NOISE_FLOOR_MIXED = 2.0 ** -44  # the double-float closures' precision
NOISE_CAP = 1e-9                # calibrated noise never exceeds this
MORE_SEEDS = 32   # added on a column that the first NSEEDS do not cover
MAX_RECHECK = 64  # columns re-measured that way, at most

# per-test parity statistics, printed in the session summary (conftest.py)
SUMMARY = []


def require_gpu():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")


def _fields(w, st, escale=None):
    """Per-cell comparison fields: vartheta_l, theta_i, rho_e_int / scale
    (escale: the scale, default max |rho_e_int| of w's initial state)."""
    out = [st[0]]
    if w.cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY:
        out.append(st[1])
        out.append(st[2] / (np.max(np.abs(w.rho_e_int)) if escale is None else escale))
    return out


def _colmax(w, a, b):
    return np.maximum.reduceat(np.abs(a - b), w.offsets[:-1].astype(np.int64))


def field_scales(w):
    """Each state field's scale: max |field| of the initial state."""
    st = w.copy_state()
    return [None if a is None else float(np.max(np.abs(a))) for a in st[:3]]


def oracle_run(w, nsteps, oracle_cfg=None, perturb_seed=None, noise=None, scales=None):
    """The oracle; with perturb_seed, random noise of size `noise` (relative
    to each field's scale; default 1 ulp: the rounding differences an
    independent FP64 implementation makes every step; a scalar or one value
    per column) is added to every nonzero state value before each step.
    scales: the fields' scales (default field_scales(w))."""
    o = O.Oracle(w)
    if oracle_cfg:
        o.set_cfg(**oracle_cfg)
    st = w.copy_state()
    if perturb_seed is None:
        rc, fl, it = o.step(st, w.t0, w.dt, nsteps)
        assert rc == 0, rc
        return st, fl, it
    rng = np.random.default_rng(perturb_seed)
    eps = np.finfo(np.float64).eps if noise is None else noise
    if np.ndim(eps):
        eps = np.repeat(np.asarray(eps, np.float64), w.nlayers)
    scale = field_scales(w) if scales is None else scales
    for k in range(nsteps):
        for i in (0, 1, 2):
            if st[i] is not None:
                st[i][:] = st[i] + (st[i] != 0.0) * (eps * scale[i]) * rng.choice([-1.0, 1.0], st[i].shape)
        rc, fl, it = o.step(st, w.t0 + k * w.dt, w.dt, 1)
    return st, fl, it


def oracle_spread(w, nsteps, ref_state, oracle_cfg=None, nseeds=NSEEDS, noise=None, seeds=None,
                  scales=None, escale=None):
    """Per-column max difference between the oracle and its perturbed runs:
    of each state field, and of the water and energy budget defects.
    seeds: the seeds (default range(nseeds)); scales, escale: the noise and
    comparison scales of the workload w was cut from (default w's own)."""
    ref = _fields(w, ref_state, escale)
    spread = [np.zeros(w.ncol) for _ in ref]
    bref = budget_defects(w, w.copy_state(), ref_state, *O.Oracle(w).budgets(ref_state))
    bspread = [np.zeros(w.ncol), np.zeros(w.ncol)]
    for seed in (range(nseeds) if seeds is None else seeds):
        st, _, _ = oracle_run(w, nsteps, oracle_cfg, perturb_seed=seed, noise=noise, scales=scales)
        for i, f in enumerate(_fields(w, st, escale)):
            spread[i] = np.maximum(spread[i], _colmax(w, ref[i], f))
        b = budget_defects(w, w.copy_state(), st, *O.Oracle(w).budgets(st))
        for i in (0, 1):
            bspread[i] = np.maximum(bspread[i], np.abs(b[i] - bref[i]))
    return spread, bspread


def step_deviation(w, nsteps, oracle_cfg=None, every=4, **dev_kw):
    """Per column, the largest one-step difference (the parity fields) between
    the GPU and the oracle, each stepping from the oracle's state, at every
    `every`-th step of the oracle's trajectory."""
    o = O.Oracle(w)
    if oracle_cfg:
        o.set_cfg(**oracle_cfg)
    st = w.copy_state()
    dev = np.zeros(w.ncol)
    with D.SoilColumns(w, **dev_kw) as g:
        for k in range(nsteps):
            t = w.t0 + k * w.dt
            sg = None
            if k % every == 0:
                g.set_state(*[None if a is None else a.copy() for a in st])
                g.step(t, w.dt, 1)
                sg = g.get_state()
            rc, _, _ = o.step(st, t, w.dt, 1)
            assert rc == 0, rc
            if sg is not None:
                for a, b in zip(_fields(w, st), _fields(w, sg)):
                    dev = np.maximum(dev, _colmax(w, a, b))
    return dev


def gpu_run(w, nsteps, **dev_kw):
    with D.SoilColumns(w, **dev_kw) as g:
        g.step(w.t0, w.dt, nsteps)
        sg = g.get_state()
        fg, ig = g.status()
        Wg, Eg = g.budgets()
    return sg, fg, ig, Wg, Eg


def check_parity(w, nsteps, oracle_cfg=None, spread=True, tol_state=TOL_STATE, noise=None,
                 nseeds=NSEEDS, name=None, **dev_kw):
    """Run the oracle and the GPU on the same workload and apply the
    criterion above. noise: None (1 ulp), a relative size, or "calibrated"
    (each column's own one-step difference, the mixed path). Returns a
    stats dict, also kept in SUMMARY."""
    so, fo, io = oracle_run(w, nsteps, oracle_cfg)
    sg, fg, ig, Wg, Eg = gpu_run(w, nsteps, **dev_kw)
    ref, got = _fields(w, so), _fields(w, sg)
    errs = [_colmax(w, r, g) for r, g in zip(ref, got)]
    names = ["vartheta_l", "theta_i", "rho_e_int_rel"][: len(errs)]
    noise_desc = "1 ulp" if noise is None else (noise if isinstance(noise, str) else f"{noise:.3g}")
    if isinstance(noise, str) and noise == "calibrated":
        dev = step_deviation(w, nsteps, oracle_cfg, **dev_kw)
        noise = np.clip(dev, NOISE_FLOOR_MIXED, NOISE_CAP)
    if spread:
        spr, bspr = oracle_spread(w, nsteps, so, oracle_cfg, nseeds=nseeds, noise=noise)
    else:
        spr = [np.zeros(w.ncol) for _ in errs]
        bspr = [np.zeros(w.ncol), np.zeros(w.ncol)]
    rechecked = _more_seeds(w, nsteps, so, errs, spr, bspr, tol_state, oracle_cfg, noise, nseeds) if spread else 0
    total_spread = np.max(np.stack(spr), axis=0)
    sensitive = total_spread > SENSITIVE
    oracle_self = float(np.mean(total_spread > tol_state))
    stats = {"columns": w.ncol, "steps": nsteps, "noise": noise_desc, "seeds": nseeds,
             "sensitive": int(sensitive.sum()), "rechecked": rechecked,
             "oracle_self_excused_frac": oracle_self}
    excused = np.zeros(w.ncol, bool)
    for nm, e, sp in zip(names, errs, spr):
        excused |= e > tol_state
        allowed = np.maximum(tol_state, SPREAD_FACTOR * sp)
        stats[f"{nm}_max_err_insensitive"] = float(e[~sensitive].max()) if (~sensitive).any() else 0.0
        stats[f"{nm}_max_err_all"] = float(e.max())
        bad = e > allowed
        assert not bad.any(), (
            f"{w.name}: {nm} error {e[bad].max():.3e} exceeds max({tol_state:g}, {SPREAD_FACTOR:g} x "
            f"oracle spread) on columns {np.nonzero(bad)[0][:8]} "
            f"(spread {sp[bad][:4]}, error {e[bad][:4]})")
    stats["excused"] = int(excused.sum())
    stats["excused_frac"] = float(excused.mean())
    total_err = np.max(np.stack(errs), axis=0)
    ratio = total_err[excused] / np.maximum(total_spread[excused], 1e-300)
    stats["excused_err_over_spread_max"] = float(ratio.max()) if excused.any() else 0.0
    SUMMARY.append((name or w.name, stats))
    assert excused.mean() <= max(MAX_SENSITIVE, oracle_self), stats
    err_fw = float(np.max(np.abs(so[3] - sg[3])) / max(np.max(np.abs(so[3])), 1e-30))
    stats["intF_w_rel"] = err_fw
    bg = budget_defects(w, w.copy_state(), sg, Wg, Eg)
    bo = budget_defects(w, w.copy_state(), so, *O.Oracle(w).budgets(so))
    stats.update(budget_water=float(bg[0].max()), budget_energy=float(bg[1].max()),
                 oracle_budget_water=float(bo[0].max()), oracle_budget_energy=float(bo[1].max()))
    for nm, g, o, sp in zip(("water", "energy"), bg, bo, bspr):
        allowed = np.maximum(1e-8 * o + 1e-12, SPREAD_FACTOR * sp)
        bad = (g >= TOL_BUDGET) & (np.abs(g - o) > allowed)
        assert not bad.any(), (nm, np.nonzero(bad)[0][:8], g[bad][:4], o[bad][:4], stats)
    stats["oracle_iters_max"] = int(io.max())
    stats["gpu_iters_max"] = int(ig.max())
    stats["iters_agree"] = float(np.mean(io == ig))
    stats["gpu_flags"] = int(np.bitwise_or.reduce(fg)) if fg.size else 0
    return stats


def _more_seeds(w, nsteps, so, errs, spr, bspr, tol_state, oracle_cfg, noise, nseeds):
    """Columns whose error the first seeds' spread does not cover get
    MORE_SEEDS further perturbed runs, each column on its own (the workload's
    noise and comparison scales kept); spr and bspr are raised in place.
    Returns how many columns were re-measured."""
    uncovered = np.any([e > np.maximum(tol_state, SPREAD_FACTOR * sp) for e, sp in zip(errs, spr)], axis=0)
    cols = np.nonzero(uncovered)[0]
    if len(cols) == 0 or len(cols) > MAX_RECHECK:
        return 0
    scales = field_scales(w)
    escale = float(np.max(np.abs(w.rho_e_int))) if w.rho_e_int is not None else None
    off = w.offsets.astype(np.int64)
    for c in cols:
        a, b = off[c], off[c + 1]
        ref = tuple(None if x is None else (x[a:b] if i < 3 else x[c:c + 1]).copy() for i, x in enumerate(so))
        nz = noise[c:c + 1] if np.ndim(noise) else noise
        sc, bc = oracle_spread(w.columns(c, c + 1), nsteps, ref, oracle_cfg, noise=nz,
                               seeds=range(nseeds, nseeds + MORE_SEEDS), scales=scales, escale=escale)
        for i in range(len(spr)):
            spr[i][c] = max(spr[i][c], sc[i][0])
        for i in (0, 1):
            bspr[i][c] = max(bspr[i][c], bc[i][0])
    return len(cols)


def budget_defects(w, state0, state1, W1, E1):
    """Per column |(W1 - W0) - (intF_w1 - intF_w0)| / |W0| and the same for
    energy (zeros for RichardsModel)."""
    o = O.Oracle(w)
    W0, E0 = o.budgets(state0)
    ew = np.abs((W1 - W0) - (state1[3] - state0[3])) / np.abs(W0)
    ee = np.zeros(w.ncol)
    if w.cfg.model == A.CLM_MODEL_ENERGY_HYDROLOGY:
        ee = np.abs((E1 - E0) - (state1[4] - state0[4])) / np.abs(E0)
    return ew, ee


TOL_MODE = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-12, energy_norm_scale=1e-9)

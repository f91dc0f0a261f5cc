"""The library's column code replayed on the CPU against the oracle.

tests/native/column_replay.cpp compiles the step kernels' column templates
(climaland.jl_gb300/csrc/clm_column.cuh: eh_column, richards_column) with
g++ and runs them one column at a time. This checks the column algebra
without a GPU: uniform and stretched geometry (clm_set_faces), FP64 and the
mixed path's float Jacobian. The device's own results are held to the
oracle by the GPU parity tests.

Criterion (FP64): every column within max(1e-10, 10 x the oracle's own
spread under per-step noise of 1 ulp of each field's scale on nonzero
values); mixed: the oracle's root to 1e-11 once
Newton has converged (8 iterations: the float Jacobian changes only the rate
of convergence; the closures are double-float), and over a trajectory at the
configured 3 iterations within max(1e-8, 10 x the spread under per-step
noise as large as each column's own one-step difference from the oracle).
"""
import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

import oracle as O
from climaland_gb300 import _abi as A
from climaland_gb300 import workloads as WL

REPO = Path(__file__).resolve().parents[1]
SRC = REPO / "tests" / "native" / "column_replay.cpp"
OUT = REPO / "tests" / "native" / "_build" / "libcolumn_replay.so"
_DP = ctypes.POINTER(ctypes.c_double)


def _lib():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    deps = [SRC, *(REPO / "climaland.jl_gb300" / "csrc").glob("*.cuh"), REPO / "include" / "climaland_cuda.h"]
    if not OUT.exists() or any(d.stat().st_mtime > OUT.stat().st_mtime for d in deps):
        OUT.parent.mkdir(parents=True, exist_ok=True)
        subprocess.run([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-fopenmp",
                        "-I", str(REPO / "climaland.jl_gb300" / "csrc"), "-I", str(REPO / "include"),
                        str(SRC), "-o", str(OUT)], check=True)
    return ctypes.CDLL(str(OUT))


def replay(w, nsteps, t0=None, guess=None, prev=None, **cfgkw):
    """The column code on the host: (state, flags, iterations) after nsteps.
    guess: (vartheta_l, rho_e_int) per-cell float32 Newton starting
    increments, or None; prev: (vartheta_l, rho_e_int) float64 arrays of the
    state at the previous step's start for the extrapolated guess, updated
    in place, or None."""
    L = _lib()
    cfg = A.ClmConfig.from_buffer_copy(w.cfg)
    for k, v in cfgkw.items():
        setattr(cfg, k, v)
    st = w.copy_state()
    keep = []

    def d(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return a.ctypes.data_as(_DP)

    fp = (ctypes.c_void_p * 4)()
    for slot, f in w.forcing.items():
        f = np.ascontiguousarray(f)
        keep.append(f)
        fp[slot] = f.ctypes.data
    prm = np.ascontiguousarray(w.params)
    off = np.ascontiguousarray(w.offsets, np.int32)
    ap = w.atmos_params or A.default_atmos_params()
    fl = np.zeros(w.ncol, np.uint32)
    it = np.zeros(w.ncol, np.int32)
    t = w.t0 if t0 is None else t0
    gp = [None, None]
    if guess is not None:
        g32 = [np.ascontiguousarray(g, np.float32) for g in guess]
        keep += g32
        gp = [g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) for g in g32]
    rc = L.clmr_step(ctypes.byref(cfg), ctypes.c_int(w.ncol), off.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                     d(w.z_lo), d(w.z_hi), d(w.z_faces), prm.ctypes.data_as(_DP), ctypes.c_int(prm.shape[0]), fp,
                     d(w.root), d(w.atmos), ctypes.byref(ap),
                     *[None if a is None else a.ctypes.data_as(_DP) for a in st],
                     ctypes.c_double(t), ctypes.c_double(w.dt), ctypes.c_int(nsteps),
                     fl.ctypes.data_as(ctypes.POINTER(ctypes.c_uint32)),
                     it.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)), *gp,
                     *([None, None] if prev is None else [p.ctypes.data_as(_DP) for p in prev]))
    assert rc == 0
    return st, fl, it


def _fields(w, st):
    out = [st[0]]
    if st[2] is not None:
        out += [st[1], st[2] / np.max(np.abs(w.rho_e_int))]
    return out


def _colmax(w, a, b):
    return np.maximum.reduceat(np.abs(a - b), w.offsets[:-1].astype(np.int64))


def _errors(w, so, sr):
    return np.max(np.stack([_colmax(w, a, b) for a, b in zip(_fields(w, so), _fields(w, sr))]), axis=0)


def _oracle(w, nsteps, noise=None, seed=None):
    """The oracle; with a seed, noise of size `noise` (relative to each
    field's scale; a scalar, or one value per column) on every nonzero state
    value before each step."""
    o = O.Oracle(w)
    st = w.copy_state()
    if seed is None:
        rc, _, _ = o.step(st, w.t0, w.dt, nsteps)
        assert rc == 0
        return st
    rng = np.random.default_rng(seed)
    eps = np.repeat(np.broadcast_to(noise, (w.ncol,)), w.nlayers)
    scale = [None if a is None else float(np.max(np.abs(a))) for a in w.copy_state()[:3]]
    for k in range(nsteps):
        for i in (0, 1, 2):
            if st[i] is not None:
                st[i][:] = st[i] + (st[i] != 0.0) * (eps * scale[i]) * rng.choice([-1.0, 1.0], st[i].shape)
        o.step(st, w.t0 + k * w.dt, w.dt, 1)
    return st


def step_deviation(w, nsteps, every=4, **kw):
    """Per column, the largest one-step difference between the replay and
    the oracle, each stepping from the oracle's own state, sampled along the
    oracle's trajectory."""
    st = w.copy_state()
    o = O.Oracle(w)
    dev = np.zeros(w.ncol)
    for k in range(nsteps):
        t = w.t0 + k * w.dt
        r = None
        if k % every == 0:
            x = w.columns(0, w.ncol)
            x.vartheta_l, x.theta_i, x.rho_e_int, x.intF_w, x.intF_e = [None if a is None else a.copy() for a in st]
            r, _, _ = replay(x, 1, t0=t, **kw)
        o.step(st, t, w.dt, 1)
        if r is not None:
            dev = np.maximum(dev, _errors(w, st, r))
    return dev


def _check(w, nsteps, tol, noise, nseeds=4, factor=10.0, **kw):
    so = _oracle(w, nsteps)
    sr, fl, _ = replay(w, nsteps, **kw)
    err = _errors(w, so, sr)
    assert np.all(np.isfinite(err)), w.name
    big = err > tol
    if big.any():
        if noise == "calibrated":
            # each column perturbed by its own one-step difference from the
            # oracle (at least 2^-44, at most 1e-9)
            noise = np.clip(step_deviation(w, nsteps, **kw), 2.0 ** -44, 1e-9)
        spread = np.zeros(w.ncol)
        for seed in range(nseeds):
            spread = np.maximum(spread, _errors(w, so, _oracle(w, nsteps, noise, seed)))
        bad = big & (err > factor * spread)
        assert not bad.any(), (w.name, np.nonzero(bad)[0][:8], err[bad][:4], spread[bad][:4])
    assert big.mean() <= 0.05, (w.name, int(big.sum()))
    return err


STRETCHED = {
    "eh": lambda: WL.stretched(WL.energy_hydrology_c1(ncol=256)),
    "full_scale": lambda: WL.stretched(WL.full_scale_c4(ncol=256)),
    "uneven": lambda: WL.stretched(WL.uneven_c2(ncol=256)),
    "global_domain": lambda: WL.global_eh_stretched(ncol=256),
    "richards": lambda: WL.stretched(WL.richards_c0(ncol=256)),
    "richards_benchmark": lambda: WL.richards_benchmark(ncol=256),
    "atmos_topmodel": lambda: WL.with_atmos(WL.stretched(WL.full_scale_c4(ncol=256)), runoff=A.CLM_RUNOFF_TOPMODEL),
    "roots": lambda: WL.with_root_extraction(WL.stretched(WL.full_scale_c4(ncol=256))),
    "brooks_corey": lambda: WL.brooks_corey(WL.stretched(WL.full_scale_c4(ncol=256))),
}


@pytest.mark.parametrize("name", list(STRETCHED))
def test_stretched_fp64_matches_oracle(name):
    w = STRETCHED[name]()
    _check(w, 48, 1e-10, np.finfo(np.float64).eps)


def test_uniform_faces_reproduce_the_uniform_path():
    """Faces at the uniform positions through the per-layer code give the
    uniform columns' result, to the rounding by which the faces' differences
    differ from the uniform path's (z_hi - z_lo) / n."""
    w = WL.full_scale_c4(ncol=128)
    nl = w.nlayers
    faces = np.concatenate([w.z_lo[c] + (w.z_hi[c] - w.z_lo[c]) * (np.arange(n + 1) / n) for c, n in enumerate(nl)])
    for c, n in enumerate(nl):
        faces[w.offsets[c] + c + n] = w.z_hi[c]
    ws = w.columns(0, w.ncol)
    ws.z_faces = faces
    a, _, _ = replay(w, 24)
    b, _, _ = replay(ws, 24)
    for x, y in zip(a, b):
        if x is not None:
            assert np.max(np.abs(x - y)) <= 1e-10 * max(1.0, np.max(np.abs(x)))


@pytest.mark.parametrize("name", ["eh", "full_scale", "richards", "global_domain"])
def test_stretched_mixed_converges_to_the_fp64_root(name):
    """With Newton run to convergence the mixed path's FP64 residual and
    increments give the oracle's step: one step from states along the
    oracle's trajectory, 8 fixed iterations on both. The residual's closures
    (psi, T, K) are double-float there (about 2^-44 relative), so the root
    agrees to 1e-11, not to FP64 rounding."""
    w = STRETCHED[name]()
    w.cfg.max_iters = 8
    st = w.copy_state()
    o = O.Oracle(w)
    worst = 0.0
    for k in range(24):
        t = w.t0 + k * w.dt
        x = w.columns(0, w.ncol)
        x.vartheta_l, x.theta_i, x.rho_e_int, x.intF_w, x.intF_e = [None if a is None else a.copy() for a in st]
        r, _, _ = replay(x, 1, t0=t, precision=A.CLM_PREC_MIXED)
        o.step(st, t, w.dt, 1)
        if k % 4 == 0:
            worst = max(worst, float(np.max(_errors(w, st, r))))
    assert worst <= 1e-11, worst


@pytest.mark.parametrize("name", ["eh", "full_scale", "global_domain", "richards"])
def test_stretched_mixed_trajectory_within_1e8(name):
    """Three fixed iterations: within 1e-8, or within 10 x the oracle's
    spread under per-step perturbations as large as the column's own
    one-step difference (the float Jacobian's slower convergence)."""
    w = STRETCHED[name]()
    _check(w, 48, 1e-8, "calibrated", nseeds=8, precision=A.CLM_PREC_MIXED)


def test_extrapolated_guess_in_tolerance_mode():
    """The extrapolated Newton start u_n + (u_n - u_{n-1}), its history kept
    in the step's own arrays: one call of 48 steps gives the bits of 48
    calls of one step and leaves the last step's starting state in the
    history; at tolerance 1e-8 it takes fewer Newton iterations per column
    than the plain start (2.25 against 2.55 measured) and stops within 1e-8
    of the plain solve on 99 % of the columns (either start stops within
    tolerance of the same root; a few chaotic columns amplify the
    difference)."""
    w = WL.full_scale_c4(ncol=2048, seed=3)
    kw = dict(precision=A.CLM_PREC_MIXED, newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-8,
              energy_norm_scale=1e-9)
    nsteps = 48

    def per_step(prev):
        st, its, start = list(w.copy_state()), [], None
        for s in range(nsteps):
            x = w.columns(0, w.ncol)
            x.vartheta_l, x.theta_i, x.rho_e_int, x.intF_w, x.intF_e = [None if a is None else a.copy()
                                                                        for a in st]
            start = (st[0].copy(), st[2].copy())
            r, fl, it = replay(x, 1, t0=w.t0 + s * w.dt, prev=prev, **kw)
            st = list(r)
            its.append(it)
        return st, np.array(its), start

    plain, ip, _ = per_step(None)
    prev = [w.vartheta_l.copy(), w.rho_e_int.copy()]
    ext, ie, start = per_step(prev)
    prev_fused = [w.vartheta_l.copy(), w.rho_e_int.copy()]
    fused, _, it_fused = replay(w, nsteps, prev=prev_fused, **kw)
    for a, b in zip(fused, ext):
        assert (a is None and b is None) or np.array_equal(a, b)
    assert np.array_equal(it_fused, ie[-1])
    for h, hf, s0 in zip(prev, prev_fused, start):
        assert np.array_equal(h, s0) and np.array_equal(hf, s0)
    assert ie[1:].mean() < ip[1:].mean() - 0.2, (ie[1:].mean(), ip[1:].mean())
    d = np.maximum.reduceat(np.abs(plain[0] - ext[0]), w.offsets[:-1].astype(np.int64))
    assert np.mean(d <= 1e-8) >= 0.99, float(np.mean(d <= 1e-8))


SPLIT_CASES = {
    "fp64": (lambda: WL.full_scale_c4(ncol=1024, seed=3), A.CLM_PREC_FP64, None),
    "mixed": (lambda: WL.full_scale_c4(ncol=1024, seed=3), A.CLM_PREC_MIXED, None),
    "mixed_extrapolated": (lambda: WL.full_scale_c4(ncol=1024, seed=3), A.CLM_PREC_MIXED, "prev"),
    "fp64_guess": (lambda: WL.full_scale_c4(ncol=1024, seed=3), A.CLM_PREC_FP64, "guess"),
    "atmos_topmodel": (lambda: WL.with_atmos(WL.full_scale_c4(ncol=512, seed=4), runoff=A.CLM_RUNOFF_TOPMODEL),
                       A.CLM_PREC_MIXED, None),
    "stretched_brooks_corey": (lambda: WL.brooks_corey(WL.stretched(WL.full_scale_c4(ncol=512, seed=5))),
                               A.CLM_PREC_FP64, "prev"),
}


@pytest.mark.parametrize("name", list(SPLIT_CASES))
def test_split_newton_resume_is_bitwise(name):
    """Split Newton (CLM_TOL_SPLIT): a column that has not converged after
    its second iteration is saved (the arrays the step kernel's hook copies
    to the queue and an EHNewtonCtx) and resumed from them alone, with its
    per-iteration arrays starting as NaN. Over eight one-step calls in
    tolerance mode the states, flags and iteration counts are those of one
    uninterrupted solve bit for bit: the save leaves nothing out. Covers
    FP64 and mixed, the plain, extrapolated and guessed starts, the
    atmosphere-driven boundary with TOPMODEL's sinks, stretched columns and
    Brooks-Corey."""
    make, prec, start = SPLIT_CASES[name]
    w = make()
    kw = dict(precision=prec, newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-8,
              energy_norm_scale=1e-9)
    L = _lib()

    def run(split_at):
        L.clmr_set_split(ctypes.c_int(split_at))
        try:
            st = list(w.copy_state())
            prev = [w.vartheta_l.copy(), w.rho_e_int.copy()] if start == "prev" else None
            last = None
            out = []
            for s in range(8):
                x = w.columns(0, w.ncol)
                x.vartheta_l, x.theta_i, x.rho_e_int, x.intF_w, x.intF_e = [None if a is None else a.copy()
                                                                            for a in st]
                guess = None
                if start == "guess" and last is not None:
                    guess = ((st[0] - last[0]).astype(np.float32), (st[2] - last[1]).astype(np.float32))
                last = (st[0].copy(), st[2].copy())
                r, fl, it = replay(x, 1, t0=w.t0 + s * w.dt, guess=guess, prev=prev, **kw)
                st = list(r)
                out.append((fl.copy(), it.copy()))
            return st, out
        finally:
            L.clmr_set_split(ctypes.c_int(0))

    ref, ref_steps = run(0)
    got, got_steps = run(2)
    for a, b in zip(ref, got):
        assert (a is None and b is None) or np.array_equal(a, b), name
    # a later split point saves a solve further along (norm history, restarts)
    got3, _ = run(3)
    for a, b in zip(ref, got3):
        assert (a is None and b is None) or np.array_equal(a, b), name
    deferred = restarted = 0
    for (fa, ia), (fb, ib) in zip(ref_steps, got_steps):
        assert np.array_equal(fa, fb) and np.array_equal(ia, ib), name
        deferred += int(np.count_nonzero(ia > 2))
        restarted += int(np.count_nonzero(((fa & A.CLM_COL_GUESS_FALLBACK) > 0) & (ia > 2)))
    assert deferred > 0, name  # the resumed path ran
    if name == "mixed_extrapolated":  # guesses dropped for a restart from U, resumed after the split
        assert restarted > 0

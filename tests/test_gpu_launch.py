"""Launch machinery of the persistent step kernel: dynamic tile order, CUDA
graph replay, capture by a caller (PyTorch) and the autotuner. None of them
may change a single bit of the results: each column's arithmetic does not
depend on which warp runs it, in which order, or how the launch was issued."""
import numpy as np
import pytest

from climaland_gb300 import _abi as A
from climaland_gb300 import learned as LG
from climaland_gb300 import workloads as WL
from climaland_gb300.device import SoilColumns
from gpu_common import require_gpu

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    require_gpu()
    import torch
    return torch


def _run(w, calls, **kw):
    """Step through `calls` = [(t, nsteps), ...]; return state, flags, iters."""
    with SoilColumns(w, **kw) as g:
        for t, n in calls:
            g.step(t, w.dt, n)
        f, it = g.status()
        return g.get_state(), f, it


def _same(a, b):
    (sa, fa, ia), (sb, fb, ib) = a, b
    for x, y in zip(sa, sb):
        if x is None:
            assert y is None
            continue
        assert np.array_equal(x, y)
    assert np.array_equal(fa, fb) and np.array_equal(ia, ib)


def test_dynamic_tile_order_bitwise_equals_static(torch):
    w = WL.uneven_c2(ncol=3000, seed=11)
    calls = [(w.t0, 6)]
    for prec in (A.CLM_PREC_FP64, A.CLM_PREC_MIXED):
        _same(_run(w, calls, precision=prec, schedule=A.CLM_SCHED_STATIC),
              _run(w, calls, precision=prec, schedule=A.CLM_SCHED_DYNAMIC))


def test_graph_replay_bitwise_equals_direct_launches(torch):
    # 70 steps = launches of 64 + 6 steps; the second call replays the graph
    # with another start time
    w = WL.uneven_c2(ncol=2048, seed=12)
    calls = [(w.t0, 70), (w.t0 + 70 * w.dt, 70), (w.t0 + 140 * w.dt, 3)]
    for sched in (A.CLM_SCHED_STATIC, A.CLM_SCHED_DYNAMIC):
        _same(_run(w, calls, schedule=sched, graph=0), _run(w, calls, schedule=sched, graph=1))
    r = WL.richards_c0(ncol=512, seed=3)
    rc = [(r.t0, 5), (r.t0 + 5 * r.dt, 5)]
    _same(_run(r, rc, graph=0), _run(r, rc, graph=1))


def test_graph_replay_with_learned_guess(torch):
    # an untrained network: the guess is poor, Newton still converges and
    # the graph and direct launches give the same bits
    w = WL.learned_eval_c3(ncol=1024, seed=5)
    tr = LG.Trainer(seed=9)
    tr.set_normalization(np.zeros(LG.N_IN), np.ones(LG.N_IN), np.zeros(LG.N_OUT), np.ones(LG.N_OUT) * 1e-4)
    blob = tr.blob()
    tr.close()
    out = []
    for graph in (0, 1):
        with SoilColumns(w, learned_guess=1, graph=graph, **LG.TOL) as g:
            g.load_mlp(blob)
            g.step(w.t0, w.dt, 4)
            g.step(w.t0 + 4 * w.dt, w.dt, 4)
            f, it = g.status()
            out.append((g.get_state(), f, it))
    _same(*out)


def test_caller_capture_records_plain_launches(torch):
    # a host that captures its own stream (PyTorch here, CUDA.jl alike) gets
    # the library's launches recorded in its graph
    w = WL.uneven_c2(ncol=1024, seed=13)
    ref = _run(w, [(w.t0, 3)])
    s = torch.cuda.Stream()
    with SoilColumns(w, graph=1) as g:
        g.set_stream(s.cuda_stream)
        cg = torch.cuda.CUDAGraph()
        with torch.cuda.graph(cg, stream=s):
            g.step_async(w.t0, w.dt, 3)
        g.set_state(*w.copy_state())  # capture does not run the kernels
        cg.replay()
        torch.cuda.synchronize()
        f, it = g.status()
        got = (g.get_state(), f, it)
    _same(ref, got)


def test_autotune_restores_state_and_changes_no_result(torch):
    w = WL.uneven_c2(ncol=4096, seed=14)
    ref = _run(w, [(w.t0, 5)])
    with SoilColumns(w) as g:
        before = g.get_state()
        table = g.autotune(w.t0, w.dt, probe_steps=2)
        assert len(table) >= 2
        assert sum(e["chosen"] for e in table) == 1
        best = min(table, key=lambda e: e["ms_per_step"])
        assert best["chosen"] == 1
        cfg = g.launch_config()
        assert (cfg["cols_per_cta"], cfg["schedule"], cfg["grid"]) == (
            best["cols_per_cta"], best["schedule"], best["grid"])
        for x, y in zip(before, g.get_state()):
            assert x is None or np.array_equal(x, y)
        g.step(w.t0, w.dt, 5)
        f, it = g.status()
        got = (g.get_state(), f, it)
    _same(ref, got)


def test_column_ranges_with_offset_equal_the_whole(torch):
    # the multi-GPU split on one device: two handles over [0, 500) and
    # [500, 1024) (column_offset keeps the rain-pulse hash global) give the
    # whole run's bits
    w = WL.full_scale_c4(ncol=1024, seed=6)
    whole = _run(w, [(w.t0, 10)])
    parts = [_run(w.columns(a, b), [(w.t0, 10)]) for a, b in ((0, 500), (500, 1024))]
    for i in range(5):
        if whole[0][i] is None:
            continue
        assert np.array_equal(whole[0][i], np.concatenate([p[0][i] for p in parts]))
    assert np.array_equal(whole[1], np.concatenate([p[1] for p in parts]))


@pytest.mark.parametrize("name,make,chunks,nsteps", [
    ("full_scale", lambda: WL.full_scale_c4(ncol=1000, seed=7), 5, 70),     # pipelined
    ("richards", lambda: WL.richards_c0(ncol=300, seed=2), 3, 4),           # pipelined
    ("uneven", lambda: WL.uneven_c2(ncol=262144, seed=8).subset(700), 4, 5),  # reorders: fallback
])
def test_host_step_equals_set_step_get(torch, name, make, chunks, nsteps):
    w = make()
    ref = _run(w, [(w.t0, nsteps)])
    st = w.copy_state()
    with SoilColumns(w, host_chunks=chunks) as g:
        g.step_host(st, w.t0, w.dt, nsteps)
        f, it = g.status()
        dev = g.get_state()
    _same(ref, (st, f, it))
    _same(ref, (dev, f, it))


@pytest.mark.parametrize("prec", [A.CLM_PREC_FP64, A.CLM_PREC_MIXED])
def test_host_step_split_newton_equals_device_step(torch, prec):
    """Tolerance mode with split Newton through the host-buffer path
    (clm_step_host: per chunk and step, the chunk's tiles then its deferred
    columns) gives the bits of the device-resident step."""
    w = WL.full_scale_c4(ncol=3000, seed=17)
    kw = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-8, energy_norm_scale=1e-9,
              precision=prec, tol_regroup=A.CLM_TOL_SPLIT)
    ref = _run(w, [(w.t0, 4)], **kw)
    st = w.copy_state()
    with SoilColumns(w, host_chunks=3, **kw) as g:
        g.step_host(st, w.t0, w.dt, 4)
        f, it = g.status()
    _same(ref, (st, f, it))
    assert int(np.count_nonzero(it > 2)) > 0


def test_atmos_boundary_graph_host_and_dynamic_paths_agree(torch):
    """The atmosphere-driven step (with TOPMODEL runoff) gives the same bits
    through direct launches, CUDA graph replay, the dynamic tile order and the
    host-buffer path (clm_step_host, pipelined chunks); drivers refreshed
    between graph-launched steps are used by the next step."""
    w = WL.with_atmos(WL.full_scale_c4(ncol=40000), runoff=A.CLM_RUNOFF_TOPMODEL)
    calls = [(w.t0, 2), (w.t0 + 2 * w.dt, 3)]
    ref = _run(w, calls, graph=0)
    _same(ref, _run(w, calls, graph=1))
    _same(ref, _run(w, calls, schedule=A.CLM_SCHED_DYNAMIC))
    st = [None if a is None else a.copy() for a in w.copy_state()]
    with SoilColumns(w, host_chunks=0) as g:
        for t, n in calls:
            g.step_host(st, t, w.dt, n)
    for x, y in zip(ref[0], st):
        assert (x is None and y is None) or np.array_equal(x, y)
    # new drivers between replays of one captured graph
    d2 = w.atmos.copy()
    d2[A.CLM_AT_T_AIR] += 3.0
    with SoilColumns(w, graph=1) as g, SoilColumns(w, graph=0) as g0:
        for h in (g, g0):
            h.step(w.t0, w.dt, 2)
            h.set_atmos(d2)
            h.step(w.t0 + 2 * w.dt, w.dt, 2)
        for x, y in zip(g.get_state(), g0.get_state()):
            assert (x is None and y is None) or np.array_equal(x, y)


@pytest.mark.parametrize("make", [lambda: WL.full_scale_c4(ncol=2000, seed=5),
                                  lambda: WL.stretched(WL.uneven_c2(ncol=2000, seed=5))])
def test_restart_from_saved_state_bitwise_equals_continuing(torch, make):
    """Checkpoint / restart as ClimaLand does it (save Y, read it back into a
    new simulation): the state read out with clm_get_state after 7 steps,
    loaded into a fresh handle with clm_set_state and stepped 5 more, gives
    the bits of one handle stepping 12; the same through the device-pointer
    entry points."""
    w = make()

    def same_state(a, b):
        for x, y in zip(a, b):
            assert (x is None and y is None) or np.array_equal(x, y)

    for prec in (A.CLM_PREC_FP64, A.CLM_PREC_MIXED):
        ref = _run(w, [(w.t0, 12)], precision=prec)[0]
        with SoilColumns(w, precision=prec) as g:
            g.step(w.t0, w.dt, 7)
            saved = g.get_state()
        wr = w.columns(0, w.ncol)
        wr.vartheta_l, wr.theta_i, wr.rho_e_int, wr.intF_w, wr.intF_e = saved
        same_state(ref, _run(wr, [(w.t0 + 7 * w.dt, 5)], precision=prec)[0])
        # device buffers (CuArray-style caller memory)
        dev = [None if a is None else torch.tensor(a, device="cuda") for a in saved]
        with SoilColumns(w, precision=prec) as g:
            g.set_state_device([None if d is None else d.data_ptr() for d in dev])
            g.step(w.t0 + 7 * w.dt, w.dt, 5)
            same_state(ref, g.get_state())


@pytest.mark.parametrize("make", [lambda: WL.full_scale_c4(ncol=3000, seed=9),
                                  lambda: WL.uneven_c2(ncol=3000, seed=9),
                                  lambda: WL.richards_c0(ncol=3000, seed=9)])
def test_tolerance_mode_regrouping_bitwise_equals_tile_order(torch, make):
    """Tolerance mode re-sorts the columns into warps by their last Newton
    iteration count after every step; the states, flags and iteration counts
    are those of the depth-sorted tiles bit for bit (direct launches and
    graph replay, FP64 and mixed)."""
    w = make()
    tol = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-8, energy_norm_scale=1e-9)
    calls = [(w.t0, 5), (w.t0 + 5 * w.dt, 3)]
    for prec in (A.CLM_PREC_FP64, A.CLM_PREC_MIXED):
        ref = _run(w, calls, precision=prec, tol_regroup=0, **tol)
        _same(ref, _run(w, calls, precision=prec, tol_regroup=1, **tol))
        _same(ref, _run(w, calls, precision=prec, tol_regroup=1, graph=1, **tol))
        _same(ref, _run(w, calls, precision=prec, tol_regroup=1, schedule=A.CLM_SCHED_DYNAMIC, **tol))
        # split Newton: the unconverged columns finish in a second launch
        for kw in (dict(), dict(graph=1), dict(schedule=A.CLM_SCHED_DYNAMIC, cols_per_cta=128)):
            _same(ref, _run(w, calls, precision=prec, tol_regroup=A.CLM_TOL_SPLIT, **kw, **tol))


@pytest.mark.parametrize("prec", [A.CLM_PREC_FP64, A.CLM_PREC_MIXED])
def test_extrapolated_guess_bitwise_over_launch_shapes(torch, prec):
    """CLM_GUESS_EXTRAPOLATE keeps its history in the handle: one call of 12
    steps (one fused launch), twelve calls of one step, graph replay and
    warp regrouping give the same bits; a state round trip through host
    buffers between calls keeps the history."""
    w = WL.full_scale_c4(ncol=3000, seed=5)
    tol = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-8, energy_norm_scale=1e-9,
               learned_guess=A.CLM_GUESS_EXTRAPOLATE, precision=prec)
    ones = [(w.t0 + i * w.dt, 1) for i in range(12)]
    ref = _run(w, [(w.t0, 12)], tol_regroup=0, **tol)
    # flags cover a call's steps: the last one-step call's are a subset of
    # the twelve-step call's
    for kw in (dict(tol_regroup=0), dict(tol_regroup=1), dict(tol_regroup=1, graph=1),
               dict(tol_regroup=A.CLM_TOL_SPLIT), dict(tol_regroup=A.CLM_TOL_SPLIT, graph=1)):
        got = _run(w, ones, **kw, **tol)
        _same(ref, (got[0], got[1] | ref[1], got[2]))
    # a twelve-step call under split Newton: twelve step pairs, the same bits
    _same(ref, _run(w, [(w.t0, 12)], tol_regroup=A.CLM_TOL_SPLIT, **tol))
    with SoilColumns(w, tol_regroup=1, **tol) as g:
        for t, n in ones:
            g.step(t, w.dt, n)
            g.set_state(*g.get_state())
        f, it = g.status()
        _same(ref, (g.get_state(), f | ref[1], it))


@pytest.mark.parametrize("make", [
    lambda: WL.stretched(WL.full_scale_c4(ncol=2000, seed=12)),
    lambda: WL.brooks_corey(WL.full_scale_c4(ncol=2000, seed=13)),
    lambda: WL.brooks_corey(WL.stretched(WL.uneven_c2(ncol=2000, seed=14))),
    lambda: WL.with_atmos(WL.full_scale_c4(ncol=2000, seed=15), runoff=A.CLM_RUNOFF_TOPMODEL),
    lambda: WL.with_root_extraction(WL.full_scale_c4(ncol=2000, seed=16)),
])
def test_split_newton_bitwise_across_kernel_variants(torch, make):
    """Split Newton on every step-kernel variant that defers (per-layer
    geometry, Brooks-Corey, the atmosphere-driven boundary with TOPMODEL's
    sinks, root extraction) and the resuming kernel of each closure and
    geometry: the states, flags and iteration counts of the depth-sorted
    tiles bit for bit, FP64 and mixed, from U and from the extrapolated
    start."""
    w = make()
    tol = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-8, energy_norm_scale=1e-9)
    ones = [(w.t0 + i * w.dt, 1) for i in range(6)]
    for prec in (A.CLM_PREC_FP64, A.CLM_PREC_MIXED):
        for guess in (A.CLM_GUESS_NONE, A.CLM_GUESS_EXTRAPOLATE):
            kw = dict(tol, precision=prec, learned_guess=guess)
            ref = _run(w, ones, tol_regroup=A.CLM_TOL_TILES, **kw)
            got = _run(w, ones, tol_regroup=A.CLM_TOL_SPLIT, **kw)
            _same(ref, got)
            assert int(np.count_nonzero(ref[2] > 2)) > 0  # the resuming kernel ran

"""Benchmark of the fused soil column step on GB300.

python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                [--config c4] [--precision fp64|mixed] [--ncol NCOL] [--top flux|atmos]

--top atmos runs the same columns under the atmosphere-driven top boundary
(turbulent fluxes, radiation, sublimation) with seeded per-column drivers.

Workload (default): the full-scale EnergyHydrology configuration,
1,048,576 columns x 20 layers (depth 1-5 m, diurnal heat flux, rain pulses,
advective heat), seeded synthetic inputs. A step is one IMEX ARS111 step of
every column (explicit stage, 3 Newton iterations, block Thomas solves),
launched as one kernel that reads and writes the whole state in HBM
(503 MB of state, larger than L2, so no flush is needed between steps).

Prints one JSON line (rank 0). Metric: column-steps/s.
  value     device-timed throughput, state resident in HBM (CUDA events on
            the library's stream, max over ranks)
  e2e       the same through the C ABI with host buffers (clm_step_host,
            wall clock): per step the state is copied in from pinned host
            memory, stepped, and copied back, pipelined over column chunks
  roofline  dominant kernel (the step kernel) against the measured HBM peak
  compute_bound  the FP64 pipe's busy fraction for that kernel (committed ncu capture)
  cpu_baseline  the FP64 CPU oracle on a bounded sample, all host threads
  forms     mixed precision, uneven columns, learned guess and the
            atmosphere-driven boundary on 262,144-column subsets
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "climaland.jl_gb300"))

import numpy as np  # noqa: E402


def algorithmic_bytes_per_column_step(model: int, nlayers: float) -> float:
    """Unavoidable HBM traffic of one column-step with the state read and
    written once. EnergyHydrology: 3 state arrays in + out (48 n) + intF_w,
    intF_e in + out (32) + 13 parameters (104) + forcing (16) + geometry (16)
    = 48 n + 168 bytes. Richards: 16 n + 16 + 48 + 8 + 8 = 16 n + 80."""
    if model == 1:
        return 48.0 * nlayers + 168.0
    return 16.0 * nlayers + 80.0


class ClockSampler:
    """Samples SM clock and throttle reasons with nvidia-smi during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev_id: str | None):
        self.dev_id = dev_id
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def __enter__(self):
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.dev_id:
            cmd += ["-i", self.dev_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self._t:
                self._t.join(timeout=2)

    def summary(self) -> dict:
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[4:8]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax),
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_traffic(kernel_key: str) -> dict | None:
    """DRAM bytes per launch of the step kernel from the committed ncu
    summary (profiles/<kernel_key>.json), if present."""
    p = REPO / "profiles" / f"{kernel_key}.json"
    if p.exists():
        return json.loads(p.read_text())
    return None


def make_workload(name: str, ncol: int | None, rank: int, top: str = "flux"):
    from climaland_gb300 import workloads as WL

    gen = WL.CONFIGS[name]
    kw = {"seed": rank}
    if ncol:
        kw["ncol"] = ncol
    w = gen(**kw)
    if top == "atmos":  # the atmosphere-driven top boundary on the same columns
        w = WL.with_atmos(w, seed=rank)
    # rank r holds columns [r ncol, (r + 1) ncol) of one domain: the
    # rain-pulse hash sees global column indices
    w.cfg.column_offset = rank * w.ncol
    return w


def cpu_baseline(w, sample_cols: int, sample_steps: int) -> dict:
    """The FP64 oracle (C, OpenMP) on a bounded sample of the workload."""
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle as O

    sub = w.subset(sample_cols)
    threads = os.cpu_count() or 1
    o = O.Oracle(sub, nthreads=threads)
    st = sub.copy_state()
    o.step(st, sub.t0, sub.dt, 1)  # warm-up (thread pool, page faults)
    st = sub.copy_state()
    t0 = time.perf_counter()
    rc, _, _ = o.step(st, sub.t0, sub.dt, sample_steps)
    el = time.perf_counter() - t0
    return {"value": sub.ncol * sample_steps / el, "unit": "column-steps/s", "cores": threads,
            "kind": "port",
            "sample": f"{sub.ncol} of {w.ncol} columns x {sample_steps} steps, FP64 oracle "
                      f"(C/OpenMP restatement; the Julia reference does not run here)",
            "seconds": el}


def run_reference(args, rank, world):
    """--impl reference: the reference's CPU path (the oracle port; Julia is
    absent) on the host cores, same config and metric."""
    if rank != 0:
        return
    w = make_workload(args.config, args.ncol, 0, args.top)
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle as O

    sample = min(w.ncol, args.ref_sample_cols)
    sub = w.subset(sample)
    threads = os.cpu_count() or 1
    o = O.Oracle(sub, nthreads=threads)
    st = sub.copy_state()
    t = sub.t0
    for _ in range(args.warmup):
        o.step(st, t, sub.dt, 1)
        t += sub.dt
    t0 = time.perf_counter()
    for _ in range(args.steps):
        o.step(st, t, sub.dt, 1)
        t += sub.dt
    el = time.perf_counter() - t0
    value = sub.ncol * args.steps / el
    line = {
        "impl": "reference", "metric": "column-steps/s", "value": value, "unit": "column-steps/s",
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": w.name, "columns_timed": sub.ncol, "layers": int(w.nlayers.max())},
        "cpu_baseline": {"value": value, "unit": "column-steps/s", "cores": threads, "kind": "port",
                         "sample": f"{sub.ncol} of {w.ncol} columns per step"},
        "e2e": {"value": value, "unit": "column-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


_ORACLE_REF = {}


def _oracle_reference(w, nsteps, sample_cols, oracle_cfg, nseeds):
    """The FP64 oracle (the checker) on the first `sample_cols` columns of w
    after `nsteps` steps, and each column's spread: the largest difference
    from its runs under per-step noise of 1 ulp of each field's scale on
    nonzero values (nseeds seeds). Kept per workload and oracle settings, so
    forms that share them share one oracle run."""
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle as O

    key = (w.name, w.ncol, nsteps, sample_cols, nseeds, tuple(sorted((oracle_cfg or {}).items())))
    if key in _ORACLE_REF:
        return _ORACLE_REF[key]
    sub = w.subset(sample_cols)
    o = O.Oracle(sub)
    if oracle_cfg:
        o.set_cfg(**oracle_cfg)
    ref = sub.copy_state()
    o.step(ref, sub.t0, sub.dt, nsteps)
    off = sub.offsets[:-1].astype(np.int64)
    eh = ref[2] is not None
    scale = float(np.max(np.abs(sub.rho_e_int))) if eh else 1.0

    def fields(st):
        return [st[0]] + ([st[1], st[2] / scale] if eh else [])

    spread = np.zeros(sub.ncol)
    eps = np.finfo(np.float64).eps
    scl = [None if a is None else float(np.max(np.abs(a))) for a in sub.copy_state()[:3]]
    for seed in range(nseeds):
        rng = np.random.default_rng(seed)
        st = sub.copy_state()
        for k in range(nsteps):
            for i in (0, 1, 2):
                if st[i] is not None:
                    st[i][:] = st[i] + (st[i] != 0.0) * (eps * scl[i]) * rng.choice([-1.0, 1.0], st[i].shape)
            o.step(st, sub.t0 + k * sub.dt, sub.dt, 1)
        sp = [np.maximum.reduceat(np.abs(a - b), off) for a, b in zip(fields(ref), fields(st))]
        spread = np.maximum(spread, np.max(np.stack(sp), axis=0))
    r = (sub, fields(ref), fields, off, spread)
    _ORACLE_REF[key] = r
    return r


def oracle_errors(w, state, nsteps, sample_cols, oracle_cfg=None, nseeds=8):
    """The form's error against the FP64 oracle (the checker) on the first
    `sample_cols` columns: max |vartheta_l|, |theta_i| and |rho_e_int| /
    max |rho_e_int| differences after `nsteps` steps, the fraction of
    columns within 1e-8 and 1e-10 in vartheta_l, and how many columns are
    above 1e-10 in any field, of which how many lie within 10 x the oracle's
    own spread under per-step noise of 1 ulp of each field's scale on nonzero
    values (8 seeds) -- the parity tests' criterion -- and on how many
    columns the oracle's own perturbed runs exceed 1e-10."""
    sub, ref, fields, off, spread = _oracle_reference(w, nsteps, sample_cols, oracle_cfg, nseeds)
    n = sub.ncells
    got = [None if a is None else a[:n] for a in state[:3]]
    eh = len(ref) > 1
    colerr = [np.maximum.reduceat(np.abs(a - b), off) for a, b in zip(ref, fields(got))]
    tot = np.max(np.stack(colerr), axis=0)
    above = tot > 1e-10
    out = {"sample_cols": sub.ncol, "steps": nsteps,
           "vartheta_l_max_abs": float(colerr[0].max()),
           "frac_cols_le_1e-8": float(np.mean(colerr[0] <= 1e-8)),
           "frac_cols_le_1e-10": float(np.mean(colerr[0] <= 1e-10)),
           "cols_above_1e-10": int(above.sum()),
           "of_which_within_10x_oracle_spread": int(np.sum(above & (tot <= 10.0 * spread))),
           "oracle_itself_above_1e-10": int(np.sum(spread > 1e-10))}
    if eh:
        out["theta_i_max_abs"] = float(colerr[1].max())
        out["rho_e_int_max_rel"] = float(colerr[2].max())
    if oracle_cfg:
        out["oracle_newton"] = dict(oracle_cfg)
    return out


def _error_stats(a, b, ncol_cells):
    """Per-column max |vartheta_l| difference statistics of state a vs b."""
    d = np.abs(a[0] - b[0])
    off = ncol_cells
    col = np.maximum.reduceat(d, off[:-1]) if len(off) > 1 else d
    return {"max_abs": float(col.max()), "q99": float(np.quantile(col, 0.99)),
            "q999": float(np.quantile(col, 0.999)),
            "frac_cols_le_1e-8": float(np.mean(col <= 1e-8)),
            "frac_cols_le_1e-10": float(np.mean(col <= 1e-10))}


def forms_block(args, torch, stream):
    """The three forms beside the plain path, on subsets that finish in
    seconds: mixed precision (EnergyHydrology and RichardsModel), uneven
    columns (autotuned, graph-replayed) and learned guess + mixed precision in
    tolerance mode; stretched columns (the reference RichardsModel
    benchmark's geometry and Newton settings, EnergyHydrology on the global
    domain's column); and the atmosphere-driven top boundary's cost on the
    full-scale columns. Each form reports err_vs_plain_fp64 (per-column max
    |vartheta_l| differences from the plain FP64 path on the same columns and
    steps) and err_vs_oracle (the FP64 oracle, as the checker, on the first
    --oracle-cols columns)."""
    from climaland_gb300 import _abi as A
    from climaland_gb300 import device as D
    from climaland_gb300 import learned as LG
    from climaland_gb300 import workloads as WL

    nst = args.forms_steps
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)

    def run(w, tune=True, blob=None, **kw):
        with D.SoilColumns(w, **kw) as g:
            g.set_stream(stream.cuda_stream)
            if tune:
                g.autotune(w.t0, w.dt, probe_steps=2)
            if blob is not None:
                g.load_mlp(blob)
            its = []
            t = w.t0
            for _ in range(nst):  # untimed pass: state, iterations, flags
                g.step(t, w.dt, 1)
                t += w.dt
                f, it = g.status()
                its.append(it)
            state = g.get_state()
            g.set_state(*w.copy_state())
            if blob is not None:
                g.load_mlp(blob)  # restarts the guess history at the initial state
            g.step(w.t0, w.dt, nst)  # same call as timed: captures its graph if any
            g.set_state(*w.copy_state())
            if blob is not None:
                g.load_mlp(blob)
            torch.cuda.synchronize()
            e0.record(stream)
            g.step_async(w.t0, w.dt, nst)
            e1.record(stream)
            stream.synchronize()
            ms = e0.elapsed_time(e1) / nst
            its = np.asarray(its, np.float64)
            return {"state": state, "ms_per_step": ms, "value": w.ncol / ms * 1e3,
                    "newton_iters_mean": float(its.mean()),
                    "fallback_frac": float(np.mean((f & A.CLM_COL_GUESS_FALLBACK) > 0)),
                    "launch_config": g.launch_config()}

    def pub(r, base, w, oracle_cfg=None):
        out = {k: v for k, v in r.items() if k != "state"}
        out["unit"] = "column-steps/s"
        if base is not None:
            out["speedup_vs_plain_fp64"] = r["value"] / base["value"]
            out["err_vs_plain_fp64"] = _error_stats(r["state"], base["state"], w.offsets)
        if args.oracle_cols > 0:
            out["err_vs_oracle"] = oracle_errors(w, r["state"], nst, args.oracle_cols, oracle_cfg)
        return out

    out = {"steps": nst}
    # full-scale distribution, 20 layers
    w4 = WL.full_scale_c4(ncol=args.forms_ncol, seed=0)
    plain = run(w4)
    mixed = run(w4, precision=A.CLM_PREC_MIXED)
    out["full_scale_subset"] = {"workload": w4.name, "plain_fp64": pub(plain, None, w4),
                                "mixed": pub(mixed, plain, w4)}
    # (1)+(4) learned guess + mixed precision, tolerance-stopped Newton:
    # network trained on the plain solver's trajectories (another seed)
    tol = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-8, energy_norm_scale=1e-9)
    wtr = WL.full_scale_c4(ncol=65536, seed=7)
    t0 = time.perf_counter()
    X, Y = LG.generate(wtr, 32, newton=tol)  # trajectories at the evaluated tolerance
    # the network as trained (no validation gate), to show what it adds
    res = LG.train(X, Y, steps=20000, batch=4096, lr=2e-3, gate=False)
    gen_train_s = time.perf_counter() - t0
    del X, Y
    # the library's default schedule (CLM_TOL_AUTO): FP64 from U regrouped by
    # iteration count, everything else split Newton (two iterations for every
    # column, then the unconverged columns packed 32 to a warp); beside them
    # the other schedules (the same bits)
    mxt = dict(tol, precision=A.CLM_PREC_MIXED)
    plain_tol = run(w4, **tol)
    plain_split = run(w4, tol_regroup=A.CLM_TOL_SPLIT, **tol)
    mixed_tol = run(w4, **mxt)
    mixed_regroup = run(w4, tol_regroup=A.CLM_TOL_REGROUP, **mxt)
    learned = run(w4, blob=res.blob, learned_guess=1, **mxt)
    # the previous increment alone (the network's output held at zero)
    persist = run(w4, blob=LG.zero_change_blob(), learned_guess=1, **mxt)
    # the same start computed inside the step kernel (no network launch)
    extrap = run(w4, learned_guess=A.CLM_GUESS_EXTRAPOLATE, **mxt)
    extrap_tiles = run(w4, learned_guess=A.CLM_GUESS_EXTRAPOLATE, tol_regroup=A.CLM_TOL_TILES, **mxt)
    fs = out["full_scale_subset"]
    fs["plain_fp64_tol1e-8"] = pub(plain_tol, plain, w4, tol)
    fs["plain_fp64_tol1e-8_split"] = pub(plain_split, plain, w4, tol)
    fs["mixed_tol1e-8"] = pub(mixed_tol, plain, w4, tol)
    fs["mixed_tol1e-8_regroup"] = pub(mixed_regroup, plain, w4, tol)
    fs["learned_mixed_tol1e-8"] = pub(learned, plain, w4, tol)
    fs["previous_increment_mixed_tol1e-8"] = pub(persist, plain, w4, tol)
    fs["extrapolated_mixed_tol1e-8"] = pub(extrap, plain, w4, tol)
    fs["extrapolated_mixed_tol1e-8_tiles"] = pub(extrap_tiles, plain, w4, tol)
    fs["tolerance_schedules"] = ("default CLM_TOL_AUTO: FP64 from U regrouped by iteration count, the "
                                 "others split Newton; _split, _regroup, _tiles: that schedule forced")
    out["full_scale_subset"]["learned_training"] = {
        "pairs": res.nrows, "train_steps": 20000, "loss_first": float(res.loss[:50].mean()),
        "loss_last": float(res.loss[-200:].mean()), "train_s": res.seconds, "gen_train_s": gen_train_s,
        "heldout_score": res.val_mse, "heldout_score_zero_change": res.val_mse_zero,
        "validation_gate_would_replace_it": bool(not res.val_mse < res.val_mse_zero),
        "heldout_metric": "mean log10 of each row's error norm in the tolerance test's terms (vartheta_l, 1e-9 rho_e_int)"}
    # (2) uneven columns, 4-30 layers, CSR: autotuned launch, CUDA graph replay
    w2 = WL.uneven_c2(ncol=args.forms_ncol, seed=0)
    u64 = run(w2, graph=1)
    umx = run(w2, graph=1, precision=A.CLM_PREC_MIXED)
    out["uneven_4_30"] = {"workload": w2.name, "cells": int(w2.ncells),
                          "plain_fp64_graph_autotuned": pub(u64, None, w2),
                          "mixed_graph_autotuned": pub(umx, u64, w2)}
    # (1) on the RichardsModel: the 1024 x 20 configuration's distributions
    w0 = WL.richards_c0(ncol=args.forms_ncol, seed=0)
    r64 = run(w0)
    rmx = run(w0, precision=A.CLM_PREC_MIXED)
    out["richards_subset"] = {"workload": w0.name, "plain_fp64": pub(r64, None, w0),
                              "mixed": pub(rmx, r64, w0)}
    # stretched columns: the reference RichardsModel benchmark
    # (experiments/benchmarks/richards.jl: 15 layers over 50 m with
    # dz_tuple = (10.0, 0.1), TOPMODEL, 2 Newton iterations, dt = 1800 s) and
    # EnergyHydrology on global_domain's column (dz_tuple = (10.0, 0.05))
    wrb = WL.richards_benchmark(ncol=args.forms_ncol, seed=0)
    rb64 = run(wrb)
    out["stretched_richards_benchmark"] = {"workload": wrb.name, "plain_fp64": pub(rb64, None, wrb)}
    wge = WL.global_eh_stretched(ncol=args.forms_ncol, seed=0)
    ge64 = run(wge)
    gemx = run(wge, precision=A.CLM_PREC_MIXED)
    out["stretched_global_domain"] = {"workload": wge.name, "plain_fp64": pub(ge64, None, wge),
                                      "mixed": pub(gemx, ge64, wge)}
    # the atmosphere-driven top boundary (turbulent fluxes, radiation,
    # sublimation) on the full-scale columns: its cost over the flux boundary
    wa = WL.with_atmos(w4)
    a64 = run(wa)
    amx = run(wa, precision=A.CLM_PREC_MIXED)
    # the full-scale workload itself: device time per step of each Newton form
    # (one step per call, as the headline line; 3 warm-up and 8 timed steps)
    wf = WL.full_scale_c4(ncol=1048576, seed=0)

    def timed(**kw):
        with D.SoilColumns(wf, **kw) as g:
            g.set_stream(stream.cuda_stream)
            g.autotune(wf.t0, wf.dt, probe_steps=2)
            t = wf.t0
            for _ in range(3):
                g.step_async(t, wf.dt, 1)
                t += wf.dt
            stream.synchronize()
            e0.record(stream)
            for _ in range(8):
                g.step_async(t, wf.dt, 1)
                t += wf.dt
            e1.record(stream)
            stream.synchronize()
            ms = e0.elapsed_time(e1) / 8
            f, it = g.status()
            return {"ms_per_step": ms, "value": wf.ncol / ms * 1e3, "unit": "column-steps/s",
                    "newton_iters_mean_last_step": float(it.mean()), "launch_config": g.launch_config()}

    mxk = dict(precision=A.CLM_PREC_MIXED)
    out["full_scale_1048576"] = {
        "workload": wf.name, "steps": 8,
        "mixed": timed(**mxk),
        "plain_fp64_tol1e-8": timed(**tol),
        "mixed_tol1e-8": timed(**mxk, **tol),
        "extrapolated_mixed_tol1e-8": timed(learned_guess=A.CLM_GUESS_EXTRAPOLATE, **mxk, **tol),
        "plain_fp64_tol1e-8_split": timed(tol_regroup=A.CLM_TOL_SPLIT, **tol),
        "extrapolated_fp64_tol1e-8": timed(learned_guess=A.CLM_GUESS_EXTRAPOLATE, **tol),
        "tolerance_schedules": "as full_scale_subset"}
    del wf
    out["atmos_boundary"] = {"workload": wa.name, "plain_fp64": pub(a64, None, wa),
                             "mixed": pub(amx, a64, wa),
                             "cost_vs_flux_boundary_fp64": a64["ms_per_step"] / plain["ms_per_step"],
                             "cost_vs_flux_boundary_mixed": amx["ms_per_step"] / mixed["ms_per_step"]}
    return out


def full_run(args, torch):
    """The full-scale configuration over its whole run: 1,048,576 x 20
    columns, 1536 steps of dt = 450 s (8 simulated days): the plain FP64 path
    (3 fixed Newton iterations, and tolerance 1e-8), the mixed path (the
    same two), and learned guess + mixed in tolerance mode with the step
    sequence replayed as CUDA graphs. Each run is timed on the device in
    calls of 64 steps (CUDA events around each call; between calls the
    flags and the last step's Newton iterations are read, so the mean
    iterations are sampled at every 64th step) and its final state compared
    with the FP64 oracle (the checker: fixed iterations, or the same
    tolerance) on the first --full-oracle-cols columns."""
    from climaland_gb300 import _abi as A
    from climaland_gb300 import device as D
    from climaland_gb300 import learned as LG
    from climaland_gb300 import workloads as WL

    w = WL.full_scale_c4(ncol=args.ncol or 1048576, seed=0)
    atmos = args.top == "atmos"
    if atmos:  # the atmosphere-driven top boundary on the same columns: FP64 and mixed
        w = WL.with_atmos(w)
    nst = w.nsteps
    chunk = 64
    stream = torch.cuda.Stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    tol = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-8, energy_norm_scale=1e-9)
    t0 = time.perf_counter()
    res = None
    if not atmos:
        wtr = WL.full_scale_c4(ncol=65536, seed=7)
        X, Y = LG.generate(wtr, 32, newton=tol)
        res = LG.train(X, Y, steps=20000, batch=4096, lr=2e-3, gate=False)  # the network as trained
        del X, Y
    train_s = time.perf_counter() - t0
    mx = dict(precision=A.CLM_PREC_MIXED)
    forms = [("plain_fp64", {}, None), ("plain_fp64_tol1e-8", dict(tol), None), ("mixed", mx, None),
             ("mixed_tol1e-8", dict(mx, **tol), None),
             ("learned_mixed_tol1e-8_graph", dict(mx, learned_guess=1, graph=1, **tol), res and res.blob),
             ("extrapolated_mixed_tol1e-8_graph",
              dict(mx, learned_guess=A.CLM_GUESS_EXTRAPOLATE, graph=1, **tol), None)] if not atmos else \
        [("plain_fp64", {}, None), ("mixed", mx, None)]
    if args.full_forms:  # a subset, the FP64 path always (the speed-ups' base)
        keep = set(args.full_forms.split(",")) | {"plain_fp64"}
        forms = [f for f in forms if f[0] in keep]
    out = {"workload": w.name, "columns": w.ncol, "steps": nst, "simulated_days": nst * w.dt / 86400.0,
           "top_boundary": "atmosphere-driven" if atmos else "flux",
           "learned_training_s": train_s,
           "learned_heldout_score": res.val_mse if res else None,
           "learned_heldout_score_zero_change": res.val_mse_zero if res else None,
           "learned_validation_gate_would_replace_it": bool(not res.val_mse < res.val_mse_zero) if res else None,
           "timing": f"device, calls of {chunk} steps"}
    for name, kw, blob in forms:
        with D.SoilColumns(w, **kw) as g:
            g.set_stream(stream.cuda_stream)
            g.autotune(w.t0, w.dt, probe_steps=2)
            if blob is not None:
                g.load_mlp(blob)
            g.step(w.t0, w.dt, chunk)  # warm-up (graph capture); the state is set again below
            g.set_state(*w.copy_state())
            if blob is not None:
                g.load_mlp(blob)  # restarts the guess history at the initial state
            torch.cuda.synchronize()
            ms = 0.0
            iters = []
            flags = np.zeros(w.ncol, np.uint32)
            for s0 in range(0, nst, chunk):
                k = min(chunk, nst - s0)
                e0.record(stream)
                g.step_async(w.t0 + s0 * w.dt, w.dt, k)
                e1.record(stream)
                stream.synchronize()
                ms += e0.elapsed_time(e1)
                f, it = g.status()
                flags |= f
                iters.append(float(it.mean()))
            state = g.get_state()
        cfg = tol if "tol" in name else None
        r = {"seconds": ms / 1e3, "column_steps_per_s": w.ncol * nst / (ms / 1e3),
             "newton_iters_mean_sampled": float(np.mean(iters)),
             "flagged_columns": int(np.count_nonzero(flags & ~np.uint32(A.CLM_COL_GUESS_FALLBACK))),
             "guess_fallback_columns": int(np.count_nonzero(flags & np.uint32(A.CLM_COL_GUESS_FALLBACK))),
             "err_vs_oracle": oracle_errors(w, state, nst, args.full_oracle_cols, cfg)}
        out[name] = r
        print(json.dumps({name: r}), file=sys.stderr, flush=True)
    base = out["plain_fp64"]["column_steps_per_s"]
    for name, _, _ in forms[1:]:
        out[name]["speedup_vs_plain_fp64"] = out[name]["column_steps_per_s"] / base
    print(json.dumps({"full_run": out}), flush=True)


def WL_full_scale(ncol, seed):
    """Training columns for the learned guess: the full-scale distributions
    with another seed than the timed columns."""
    from climaland_gb300 import workloads as WL
    return WL.full_scale_c4(ncol=ncol, seed=seed)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c4")
    ap.add_argument("--ncol", type=int, default=None)
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"])
    ap.add_argument("--newton", default="fixed", choices=["fixed", "tol"],
                    help="fixed: the configuration's 3 iterations; tol: stop at 1e-8 (at most 20)")
    ap.add_argument("--no-regroup", action="store_true",
                    help="tolerance mode without regrouping the columns into warps by iteration count")
    ap.add_argument("--split", action="store_true",
                    help="tolerance mode with split Newton: two iterations for every column, then the "
                         "unconverged columns packed 32 to a warp in a second launch")
    ap.add_argument("--guess", default="none", choices=["none", "extrapolate", "previous", "learned"],
                    help="Newton start (tolerance mode): U; the previous increment, inside the step "
                         "kernel (extrapolate) or through the network's launch with the network's "
                         "output held at zero (previous); or the previous increment + the network's "
                         "change (learned: trained at start, validation-gated)")
    ap.add_argument("--top", default="flux", choices=["flux", "atmos"],
                    help="top boundary: the workload's flux forcing, or the atmosphere-driven "
                         "boundary (EnergyHydrology)")
    ap.add_argument("--cpu-sample-cols", type=int, default=65536)
    ap.add_argument("--cpu-sample-steps", type=int, default=128)
    ap.add_argument("--ref-sample-cols", type=int, default=32768)
    ap.add_argument("--e2e-steps", type=int, default=None)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-forms", action="store_true")
    ap.add_argument("--forms-ncol", type=int, default=262144)
    ap.add_argument("--forms-steps", type=int, default=32)
    ap.add_argument("--oracle-cols", type=int, default=4096,
                    help="columns of each form checked against the FP64 oracle (0: none)")
    ap.add_argument("--full-run", action="store_true",
                    help="the full-scale configuration's whole 8-day run per form (minutes), "
                         "instead of the bench line")
    ap.add_argument("--full-oracle-cols", type=int, default=8192)
    ap.add_argument("--full-forms", default=None,
                    help="--full-run: comma-separated form names to run (default: all)")
    args = ap.parse_args()

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import torch

    dist = None
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local_rank)

    import __graft_entry__ as G

    G.build()
    from climaland_gb300 import _abi as A
    from climaland_gb300 import device as D

    if args.full_run:
        full_run(args, torch)
        return

    w = make_workload(args.config, args.ncol, rank, args.top)
    prec = A.CLM_PREC_MIXED if args.precision == "mixed" else A.CLM_PREC_FP64
    nl = float(w.nlayers.mean())
    newton = {}
    if args.newton == "tol" or args.guess != "none":
        newton = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-8, energy_norm_scale=1e-9)
    blob = None
    learned_gated = None
    if args.guess in ("previous", "learned"):
        from climaland_gb300 import learned as LG
        if args.guess == "learned":
            X, Y = LG.generate(WL_full_scale(65536, 7), 32, newton=newton)
            res = LG.train(X, Y, steps=20000, batch=4096, lr=2e-3)  # validation-gated
            del X, Y
            blob = res.blob if res.guess_mode == A.CLM_GUESS_NETWORK else None
            learned_gated = res.gated
        else:
            blob = LG.zero_change_blob()
    if newton and args.no_regroup:
        newton["tol_regroup"] = A.CLM_TOL_TILES
    if newton and args.split:
        newton["tol_regroup"] = A.CLM_TOL_SPLIT
    sched = newton.get("tol_regroup", A.CLM_TOL_AUTO) if newton else None
    if sched == A.CLM_TOL_AUTO:  # the library's rule
        sched = (A.CLM_TOL_REGROUP if w.cfg.model != 1 or (prec == A.CLM_PREC_FP64 and args.guess == "none")
                 else A.CLM_TOL_SPLIT)
    mode = A.CLM_GUESS_NETWORK if blob else (A.CLM_GUESS_EXTRAPOLATE if args.guess in ("extrapolate", "learned")
                                             else None)
    g = D.SoilColumns(w, precision=prec, learned_guess=mode, **newton)
    if blob:
        g.load_mlp(blob)
    stream = torch.cuda.Stream()
    g.set_stream(stream.cuda_stream)
    tune = None
    if not args.no_autotune:
        tune = g.autotune(w.t0, w.dt, probe_steps=2)  # the state is restored

    def barrier():
        if dist is not None:
            dist.barrier()

    # warm-up
    t = w.t0
    for _ in range(args.warmup):
        g.step_async(t, w.dt, 1)
        t += w.dt
    stream.synchronize()

    try:
        uuid = str(torch.cuda.get_device_properties(local_rank).uuid)
        dev_id = uuid if uuid.startswith("GPU-") else f"GPU-{uuid}"
    except Exception:
        dev_id = os.environ.get("CUDA_VISIBLE_DEVICES", "").split(",")[0] or None

    # ---- device-timed region: state resident in HBM ----------------------
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(dev_id) as clk:
        ev[0].record(stream)
        for i in range(args.steps):
            g.step_async(t, w.dt, 1)
            t += w.dt
            ev[i + 1].record(stream)
        stream.synchronize()
    torch.cuda.synchronize()
    barrier()
    per_launch_ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    total_ms = ev[0].elapsed_time(ev[-1])
    if dist is not None:
        tt = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        total_ms = float(tt.item())
    value = w.ncol * world * args.steps / (total_ms / 1e3)
    flags, iters = g.status()

    # ---- end to end through the C ABI with host buffers ------------------
    e2e_steps = args.e2e_steps or max(3, min(args.steps, 10))
    pinned = []
    for a in w.copy_state():
        if a is None:
            pinned.append(None)
            continue
        p = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
        p[:] = a
        pinned.append(p)
    h2d = sum(a.nbytes for a in pinned if a is not None)
    g.step_host([None if a is None else a.copy() for a in pinned], t, w.dt, 1)  # warm: streams, events
    barrier()
    torch.cuda.synchronize()
    # wall clock: clm_step_host is synchronous and spans three streams
    w0 = time.perf_counter()
    for i in range(e2e_steps):
        # clm_step_host: the state goes in from pinned host memory, is
        # stepped, and comes back in place, copies pipelined with the kernels
        g.step_host(pinned, t, w.dt, 1)
        t += w.dt
    torch.cuda.synchronize()
    wall_e2e_ms = (time.perf_counter() - w0) * 1e3
    if dist is not None:
        tt = torch.tensor([wall_e2e_ms], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        wall_e2e_ms = float(tt.item())
    e2e = w.ncol * world * e2e_steps / (wall_e2e_ms / 1e3)

    if rank != 0:
        g.close()
        if dist is not None:
            dist.destroy_process_group()
        return

    peaks = measured_peaks()
    bytes_per_launch = algorithmic_bytes_per_column_step(w.cfg.model, nl) * w.ncol
    if args.top == "atmos":  # the per-column drivers, read once per step
        bytes_per_launch += 8 * A.CLM_AT_NFIELDS * w.ncol
    avg_launch_s = statistics.mean(per_launch_ms) / 1e3
    achieved = bytes_per_launch / avg_launch_s / 1e9
    key = f"{'eh' if w.cfg.model == 1 else 'richards'}_step_{args.precision}"
    if args.top == "atmos":
        key += "_atmos"
    prof = profile_traffic(key)
    traffic = None
    if prof and prof.get("dram_bytes_per_column_step"):
        traffic = prof["dram_bytes_per_column_step"] * w.ncol
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                "peak_source": peaks["source"], "kernel": key,
                "bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_launch_s * 1e3}
    # the resource that bounds the step kernel (its HBM fraction is small by
    # arithmetic intensity): the FP64 pipe's busy fraction and FP64
    # instructions per cell-step from the committed ncu capture
    compute = None
    if prof and prof.get("fp64_pipe_pct_active"):
        compute = {"pipe": "fp64", "active_frac": prof["fp64_pipe_pct_active"] / 100.0,
                   "fp64_inst_per_cell_step": prof.get("fp64_inst_per_cell_step"),
                   "source": f"profiles/{key}.json (ncu, 262,144-column launch)"}
    cpu = None
    if not args.no_cpu_baseline:
        cpu = cpu_baseline(w, args.cpu_sample_cols, args.cpu_sample_steps)
    forms = None
    if not args.no_forms and world == 1:
        forms = forms_block(args, torch, stream)
        if w.ncol == 1048576 and w.cfg.model == 1:  # the same columns as this line's
            for r in forms["full_scale_1048576"].values():
                if isinstance(r, dict) and "value" in r:
                    r["speedup_vs_this_line"] = r["value"] / value
    line = {
        "metric": "column-steps/s", "value": value, "unit": "column-steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total_ms / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == A.CLM_PREC_FP64 else "f64+f32",
        "data": "synthetic",
        "config": {"workload": w.name, "columns_per_gpu": w.ncol, "layers": int(w.nlayers.max()),
                   "model": "EnergyHydrology" if w.cfg.model == 1 else "RichardsModel",
                   "newton": (f"fixed {w.cfg.max_iters} iterations" if not newton else
                              "tolerance 1e-8 (at most 20 iterations)" +
                              {A.CLM_TOL_TILES: ", depth-sorted tiles",
                               A.CLM_TOL_REGROUP: (", warps regrouped by iteration count" if args.guess == "none"
                                                   else ", depth-sorted tiles"),
                               A.CLM_TOL_SPLIT: ", split Newton (two iterations, then the unconverged columns "
                                                "packed 32 to a warp)"}[sched]),
                   "newton_start": {"none": "U", "extrapolate": "previous increment (in the step kernel)",
                                    "previous": "previous increment (network launch, zero output)",
                                    "learned": ("previous increment (in the step kernel: the validation gate "
                                                "dropped the network)" if learned_gated else
                                                "previous increment + network")}[args.guess],
                   "precision": args.precision,
                   "l2": "inputs larger than L2 (state 48 B x cells)", "dt_s": w.dt},
        "e2e": {"value": e2e, "unit": "column-steps/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": h2d, "steps": e2e_steps},
        # per step: the step kernel; in tolerance mode without a guess the
        # regrouping's three kernels, with split Newton the resuming kernel;
        # with the network guess, its kernel
        "gpu_launches": args.steps * (1 + (3 if sched == A.CLM_TOL_REGROUP and args.guess == "none" else 0)
                                      + (1 if sched == A.CLM_TOL_SPLIT else 0) + (1 if blob else 0)),
        "launch_config": dict(g.launch_config(), autotuned=tune is not None),
        "roofline": roofline,
        "compute_bound": compute,
        "cpu_baseline": cpu,
        "clocks": clk.summary(),
        "status": {"flagged_columns": int(np.count_nonzero(flags)),
                   "newton_iters_max": int(iters.max()),
                   "newton_iters_mean_last_step": float(iters.mean())},
        "forms": forms,
    }
    print(json.dumps(line), flush=True)
    g.close()
    if dist is not None:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()

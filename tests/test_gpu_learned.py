"""Learned Newton initial guess: the network's GPU forward/backward kernels
against the FP64 CPU restatement (oracle/mlp_oracle.py), training, the
feature kernel, and the end-to-end effect on tolerance-mode Newton."""
import json

import numpy as np
import pytest

import mlp_oracle as MO
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


def _random_problem(torch, n=512, seed=0):
    rng = np.random.default_rng(seed)
    X = rng.normal(size=(n, LG.N_IN)).astype(np.float32) * 3.0 + 1.0
    Y = rng.normal(size=(n, LG.N_OUT)).astype(np.float32) * 2.0 - 0.5
    norm = (rng.normal(size=LG.N_IN).astype(np.float32), rng.uniform(1, 4, LG.N_IN).astype(np.float32),
            rng.normal(size=LG.N_OUT).astype(np.float32), rng.uniform(1, 3, LG.N_OUT).astype(np.float32))
    return X, Y, norm


def _blocks(g):
    sizes = [80 * 64, 64, 64 * 64, 64, 64 * 40, 40]
    out, o = [], 0
    for s in sizes:
        out.append(g[o:o + s])
        o += s
    return out


def test_gradients_match_fp64_oracle(torch):
    X, Y, norm = _random_problem(torch)
    tr = LG.Trainer(seed=3)
    tr.set_normalization(*norm)
    Xd, Yd = torch.tensor(X, device="cuda"), torch.tensor(Y, device="cuda")
    g_gpu, loss_gpu = tr.gradients(Xd, Yd)
    loss_ref, g_ref, _ = MO.loss_and_grad(tr.params(), tr.normalization(), X, Y)
    assert abs(loss_gpu - loss_ref) / loss_ref < 1e-2
    for name, a, b in zip(["W1", "b1", "W2", "b2", "W3", "b3"], _blocks(g_gpu), _blocks(g_ref)):
        b = b.astype(np.float64)
        if name == "W1":  # padded input rows carry no gradient
            a, b = a.reshape(80, 64)[:67].ravel(), b.reshape(80, 64)[:67].ravel()
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))
        print(f"GRADCHECK {name} rel_l2={rel:.3e} cos={cos:.6f}")
        # BF16 activations (2^-8 relative) bound the agreement
        assert rel < 3e-2 and cos > 0.999, (name, rel, cos)


def test_predict_matches_fp64_oracle(torch):
    X, Y, norm = _random_problem(torch, n=1000, seed=1)
    tr = LG.Trainer(seed=5)
    tr.set_normalization(*norm)
    Yp = tr.predict(torch.tensor(X, device="cuda")).cpu().numpy()
    _, _, Yref = MO.loss_and_grad(tr.params(), tr.normalization(), X, Y)
    rel = np.linalg.norm(Yp - Yref) / np.linalg.norm(Yref)
    assert rel < 2e-2, rel


def test_training_fits_a_smooth_map(torch):
    rng = np.random.default_rng(2)
    n = 65536
    X = rng.normal(size=(n, LG.N_IN)).astype(np.float32)
    M = rng.normal(size=(LG.N_IN, LG.N_OUT)).astype(np.float32) / np.sqrt(LG.N_IN)
    Y = np.tanh(X @ M) + 0.1 * (X[:, :LG.N_OUT] ** 2)
    Xd, Yd = torch.tensor(X, device="cuda"), torch.tensor(Y.astype(np.float32), device="cuda")
    res = LG.train(Xd, Yd, steps=3000, batch=2048, lr=2e-3)
    print(f"TRAIN loss {res.loss[:50].mean():.4f} -> {res.loss[-50:].mean():.4f} in {res.seconds:.2f}s")
    assert res.loss[-50:].mean() < 0.2 * res.loss[:50].mean()
    # the held-out rows confirm the fit (mean log10 error norm 0.2 decades
    # or more below predicting zero): the network is kept
    assert res.val_mse < res.val_mse_zero - 0.2 and not res.gated


def test_validation_gate_drops_a_network_that_predicts_nothing(torch):
    """Targets independent of the inputs (zero-mean noise): the held-out error
    is not below predicting zero, so train returns the zero-change weights."""
    rng = np.random.default_rng(4)
    n = 32768
    X = rng.normal(size=(n, LG.N_IN)).astype(np.float32)
    Y = rng.normal(size=(n, LG.N_OUT)).astype(np.float32)
    res = LG.train(torch.tensor(X, device="cuda"), torch.tensor(Y, device="cuda"), steps=1000, batch=2048)
    assert res.gated and res.blob == LG.zero_change_blob(), (res.val_mse, res.val_mse_zero)


def test_features_kernel_matches_host(torch):
    w = WL.energy_hydrology_c1(ncol=300, nlayers=20, seed=1)
    X = torch.zeros((w.ncol, LG.N_IN), dtype=torch.float32, device="cuda")
    t = 3600.0 * 7
    with SoilColumns(w) as g:
        g.features(t, w.dt, X.data_ptr())
    X = X.cpu().numpy()
    v = w.vartheta_l.reshape(w.ncol, 20)
    ti = w.theta_i.reshape(w.ncol, 20)
    e = w.rho_e_int.reshape(w.ncol, 20)
    E = A.DEFAULT_EARTH
    nu = w.params[A.CLM_P_NU][:, None]
    thr = w.params[A.CLM_P_THETA_R][:, None]
    sq = np.sqrt(np.finfo(float).eps)
    tl = np.minimum(np.maximum(v, thr + sq), np.maximum(nu - ti, thr + sq))
    rc = w.params[A.CLM_P_RHOC_DS][:, None] + tl * E["cp_l"] * E["rho_l"] + ti * E["cp_i"] * E["rho_i"]
    T = E["T_0"] + (e + ti * E["rho_i"] * E["LH_f0"]) / rc
    assert np.allclose(X[:, :20], v, rtol=1e-6)
    assert np.allclose(X[:, 20:40], ti, rtol=1e-6, atol=1e-7)
    assert np.allclose(X[:, 40:60], T, rtol=1e-6)
    fh = w.forcing[A.CLM_BC_TOP_HEAT]
    assert np.allclose(X[:, 61], fh[A.CLM_F_AMP] * np.sin(fh[A.CLM_F_OMEGA] * t), rtol=1e-5, atol=1e-4)
    assert np.allclose(X[:, 65], np.log10(w.params[A.CLM_P_K_SAT]), rtol=1e-6)
    assert np.all(X[:, 66] == np.float32(w.dt))


def test_learned_guess_saves_newton_iterations(torch):
    """Train on the plain solver's trajectories, then solve unseen columns of
    the learned-guess evaluation configuration (65,536 x 20) to the bench's
    tolerance (1e-8) with and without the guess: fewer Newton iterations per
    column, the same answer within 1e-8 (the plain solve is the reference
    for its error). The guess is the previous increment plus the network's
    predicted change (train's validation gate keeps the network only where
    its held-out error is below that of predicting no change); the previous
    increment alone (the network's output held at zero) is measured beside
    it, and the step kernel's own extrapolation (CLM_GUESS_EXTRAPOLATE, the
    same start without the network's launch)."""
    tol = dict(LG.TOL, newton_tol=1e-8)
    wtr = LG.training_workload(ncol=16384, seed=0)
    X, Y = LG.generate(wtr, 24, newton=tol)
    res = LG.train(X, Y, steps=3000, batch=4096, lr=2e-3)
    zero_blob = LG.zero_change_blob()
    wev = LG.eval_workload(ncol=65536, seed=1)
    nsteps = 24
    out = {}
    runs = (("plain", None, None), ("learned", res.blob, A.CLM_GUESS_NETWORK),
            ("previous_increment", zero_blob, A.CLM_GUESS_NETWORK),
            ("extrapolated", None, A.CLM_GUESS_EXTRAPOLATE))
    for name, blob, mode in runs:
        with SoilColumns(wev, learned_guess=mode, **tol) as g:
            if blob:
                g.load_mlp(blob)
            iters = []
            t = wev.t0
            for i in range(nsteps):
                g.step(t, wev.dt, 1)
                t += wev.dt
                f, it = g.status()
                iters.append(it.astype(np.float64))
            out[name] = (g.get_state(), np.mean(iters), f)
    sp, ip, _ = out["plain"]
    stats = dict(train_rows=res.nrows, train_seconds=res.seconds, loss_first=float(res.loss[:50].mean()),
                 loss_last=float(res.loss[-50:].mean()), heldout_log10_err=res.val_mse,
                 heldout_log10_err_zero_change=res.val_mse_zero, gated=res.gated, iters_plain=ip)
    for name in ("learned", "previous_increment", "extrapolated"):
        sl, il, fl = out[name]
        colerr = np.max(np.abs(sp[0] - sl[0]).reshape(wev.ncol, 20), axis=1)
        stats[f"iters_{name}"] = il
        stats[f"fallback_frac_{name}"] = float(np.mean((fl & A.CLM_COL_GUESS_FALLBACK) > 0))
        stats[f"frac_cols_within_1e8_{name}"] = float(np.mean(colerr <= 1e-8))
        stats[f"max_err_{name}"] = float(colerr.max())
    print("LEARNED " + json.dumps(stats))
    for name in ("learned", "extrapolated"):
        assert stats[f"iters_{name}"] < ip, name
        assert stats[f"frac_cols_within_1e8_{name}"] >= 0.99, name
    # the in-kernel extrapolation is the zero-change network's guess in FP64
    # instead of float: the same iteration counts to within a few columns
    assert abs(stats["iters_extrapolated"] - stats["iters_previous_increment"]) < 0.02


@pytest.mark.parametrize("prec", [A.CLM_PREC_FP64, A.CLM_PREC_MIXED])
def test_network_guess_under_split_newton_is_bitwise(torch, prec):
    """The network's guess launch followed by split Newton (the step kernel,
    then the resuming kernel for the columns that have not converged after
    two iterations) gives the bits of the depth-sorted tiles, direct and
    graph-replayed: states, flags and iteration counts."""
    w = WL.full_scale_c4(ncol=3000, seed=8)
    tol = dict(LG.TOL, newton_tol=1e-8, precision=prec, learned_guess=A.CLM_GUESS_NETWORK)
    blob = LG.zero_change_blob()

    def run(**kw):
        with SoilColumns(w, **tol, **kw) as g:
            g.load_mlp(blob)
            t = w.t0
            for _ in range(6):
                g.step(t, w.dt, 1)
                t += w.dt
            g.step(t, w.dt, 4)
            f, it = g.status()
            return g.get_state(), f, it

    ref = run(tol_regroup=A.CLM_TOL_TILES)
    for kw in (dict(tol_regroup=A.CLM_TOL_SPLIT), dict(tol_regroup=A.CLM_TOL_SPLIT, graph=1)):
        got = run(**kw)
        for a, b in zip(ref[0], got[0]):
            assert (a is None and b is None) or np.array_equal(a, b)
        assert np.array_equal(ref[1], got[1]) and np.array_equal(ref[2], got[2])
    assert int(np.count_nonzero(ref[2] > 2)) > 0  # some columns resumed

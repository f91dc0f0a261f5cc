"""Learned Newton initial guess: training data from the plain solver, GPU
training with the library's own kernels, evaluation.

The network and its kernels live in libclimaland_cuda (clm_mlp_* and
clm_load_mlp); this module drives them with torch-owned device buffers.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from . import _abi as A
from . import workloads as WL
from .device import ClmError, SoilColumns, load_library

N_IN = 67
N_OUT = 40
LAYERS = 20


def _torch():
    import torch
    return torch


class Trainer:
    """clm_mlp handle: FP32 master weights + Adam on the GPU."""

    def __init__(self, seed=0, lib=None):
        self.lib = lib or load_library()
        h = ctypes.c_void_p()
        rc = self.lib.clm_mlp_create(int(seed), ctypes.byref(h))
        if rc != 0:
            raise ClmError(rc, "clm_mlp_create failed")
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.lib.clm_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_normalization(self, in_mean, in_std, out_mean, out_std):
        fp = lambda a: np.ascontiguousarray(a, np.float32).ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        arrs = [np.ascontiguousarray(a, np.float32) for a in (in_mean, in_std, out_mean, out_std)]
        rc = self.lib.clm_mlp_set_normalization(self.h, *[a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) for a in arrs])
        if rc != 0:
            raise ClmError(rc, "clm_mlp_set_normalization failed")

    def train(self, X, Y, batch, nsteps, lr, stream=0):
        loss = np.zeros(max(nsteps, 1), np.float32)
        rc = self.lib.clm_mlp_train(self.h, ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(Y.data_ptr()),
                                    X.shape[0], batch, nsteps, lr,
                                    loss.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                    ctypes.c_void_p(stream))
        if rc != 0:
            raise ClmError(rc, "clm_mlp_train failed")
        return loss[:nsteps]

    def gradients(self, X, Y):
        n = int(self.lib.clm_mlp_nparams())
        g = np.zeros(n, np.float32)
        loss = np.zeros(1, np.float32)
        rc = self.lib.clm_mlp_gradients(self.h, ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(Y.data_ptr()),
                                        X.shape[0], g.ctypes.data_as(ctypes.POINTER(ctypes.c_float)),
                                        loss.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        if rc != 0:
            raise ClmError(rc, "clm_mlp_gradients failed")
        return g, float(loss[0])

    def predict(self, X):
        torch = _torch()
        Y = torch.empty((X.shape[0], N_OUT), dtype=torch.float32, device=X.device)
        rc = self.lib.clm_mlp_predict(self.h, ctypes.c_void_p(X.data_ptr()), X.shape[0],
                                      ctypes.c_void_p(Y.data_ptr()), ctypes.c_void_p(0))
        if rc != 0:
            raise ClmError(rc, "clm_mlp_predict failed")
        torch.cuda.synchronize()
        return Y

    def blob(self) -> bytes:
        n = int(self.lib.clm_mlp_blob_bytes())
        buf = ctypes.create_string_buffer(n)
        rc = self.lib.clm_mlp_get(self.h, buf, n)
        if rc != 0:
            raise ClmError(rc, "clm_mlp_get failed")
        return buf.raw

    def load_blob(self, blob: bytes):
        buf = ctypes.create_string_buffer(bytes(blob), len(blob))
        rc = self.lib.clm_mlp_set(self.h, buf, len(blob))
        if rc != 0:
            raise ClmError(rc, "clm_mlp_set failed")

    def params(self) -> np.ndarray:
        raw = np.frombuffer(self.blob(), dtype=np.uint8)
        f = raw[16:].view(np.float32)
        return f[2 * N_IN + 2 * N_OUT:].copy()

    def normalization(self):
        raw = np.frombuffer(self.blob(), dtype=np.uint8)
        f = raw[16:].view(np.float32)
        return (f[:N_IN].copy(), f[N_IN:2 * N_IN].copy(), f[2 * N_IN:2 * N_IN + N_OUT].copy(),
                f[2 * N_IN + N_OUT:2 * N_IN + 2 * N_OUT].copy())


TOL = dict(newton_mode=A.CLM_NEWTON_TOL, max_iters=20, newton_tol=1e-12, energy_norm_scale=1e-9)


def generate(w, nsteps, newton=TOL):
    """(X, Y) pairs from the plain FP64 solver in tolerance mode: X the raw
    inputs at the start of step n, Y the change of the step's increment of
    vartheta_l and rho_e_int (20 layers each) from the previous step's,
    (u_{n+1} - u_n) - (u_n - u_{n-1}), for every column and step n >= 1
    (device tensors): the guess kernel adds the prediction to the column's
    previous increment."""
    torch = _torch()
    assert np.all(w.nlayers == LAYERS), "the network is built for 20-layer columns"
    ncol = w.ncol
    X = torch.empty((nsteps, ncol, N_IN), dtype=torch.float32, device="cuda")
    Y = torch.empty((nsteps, ncol, N_OUT), dtype=torch.float32, device="cuda")
    st = [None if a is None else torch.tensor(a, device="cuda") for a in w.copy_state()]
    ptrs = [x.data_ptr() for x in st]
    with SoilColumns(w, **newton) as g:
        t = w.t0
        inc_v = inc_e = None
        for i in range(nsteps):
            g.features(t, w.dt, X[i].data_ptr())
            prev_v = st[0].clone()
            prev_e = st[2].clone()
            g.step(t, w.dt, 1)
            g.get_state_device(ptrs)
            torch.cuda.synchronize()
            dv, de = st[0] - prev_v, st[2] - prev_e
            if inc_v is not None:
                Y[i, :, :LAYERS] = (dv - inc_v).view(ncol, LAYERS).float()
                Y[i, :, LAYERS:] = (de - inc_e).view(ncol, LAYERS).float()
            inc_v, inc_e = dv, de
            t += w.dt
    # the first step has no previous increment: its pair is not used
    return X[1:].reshape(-1, N_IN), Y[1:].reshape(-1, N_OUT)


@dataclass
class TrainResult:
    blob: bytes
    loss: np.ndarray
    nrows: int
    seconds: float
    val_mse: float = float("nan")       # held-out rows: mean log10 of the network's error norm
    val_mse_zero: float = float("nan")  # the same for a predicted change of zero
    gated: bool = False                 # blob is the zero-change network (see train)

    @property
    def guess_mode(self) -> int:
        """The clm_config.learned_guess to run with: the network, or, when the
        gate dropped it, the step kernel's own extrapolation (the same start
        as the zero-change network without its launch)."""
        return A.CLM_GUESS_EXTRAPOLATE if self.gated else A.CLM_GUESS_NETWORK


def zero_change_blob() -> bytes:
    """Weights whose prediction is a change of zero: the guess is then the
    column's previous step increment alone."""
    tr = Trainer(seed=0)
    tr.set_normalization(np.zeros(N_IN), np.ones(N_IN), np.zeros(N_OUT), np.full(N_OUT, 1e-30))
    blob = tr.blob()
    tr.close()
    return blob


def train(X, Y, steps=4000, batch=4096, lr=2e-3, seed=0, val_frac=0.05, gate=True, energy_scale=1e-9):
    """Standardise, shuffle and train with the library's kernels; returns the
    weight blob for clm_load_mlp. A fraction val_frac of the shuffled rows is
    held out; each row's error is its norm in the tolerance test's own terms
    (vartheta_l errors, and rho_e_int errors times energy_scale, the
    clm_config's energy_norm_scale), and the rows are scored by the mean of
    its log10: Newton's iteration count follows the order of magnitude of a
    column's start error, and a network that halves the large errors but
    lifts the many small ones costs iterations (a mean squared error kept
    such a network). With gate, a network whose score is not below that of
    predicting no change is replaced by the zero-change weights (the guess
    is then the previous increment; TrainResult.guess_mode says to run it as
    CLM_GUESS_EXTRAPOLATE)."""
    import time
    torch = _torch()
    gen = torch.Generator(device="cuda")
    gen.manual_seed(seed)
    perm = torch.randperm(X.shape[0], device="cuda", generator=gen)
    nval = int(X.shape[0] * val_frac)
    Xv = X[perm[:nval]].contiguous()
    Yv = Y[perm[:nval]].contiguous()
    perm = perm[nval:]
    Xs = X[perm].contiguous()
    Ys = Y[perm].contiguous()
    in_mean = Xs.mean(0).cpu().numpy()
    in_std = Xs.std(0).cpu().numpy()
    out_mean = Ys.mean(0).cpu().numpy()
    out_std = np.maximum(Ys.std(0).cpu().numpy(), 1e-12)
    tr = Trainer(seed=seed)
    tr.set_normalization(in_mean, in_std, out_mean, out_std)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    losses = []
    done = 0
    while done < steps:
        k = min(1000, steps - done)
        # later chunks with a decayed rate
        frac = done / max(steps, 1)
        losses.append(tr.train(Xs, Ys, batch, k, lr * (0.1 ** frac)))
        done += k
    el = time.perf_counter() - t0
    blob = tr.blob()
    val = zero = float("nan")
    if nval > 0:
        P = tr.predict(Xv)
        w = torch.ones(N_OUT, device=Yv.device)
        w[LAYERS:] = energy_scale ** 2
        val = float(torch.log10((((P - Yv) ** 2) * w).sum(1).sqrt() + 1e-30).mean())
        zero = float(torch.log10(((Yv ** 2) * w).sum(1).sqrt() + 1e-30).mean())
    tr.close()
    gated = bool(gate and nval > 0 and not val < zero)
    if gated:
        blob = zero_change_blob()
    loss = np.concatenate(losses) / (batch * N_OUT)
    return TrainResult(blob=blob, loss=loss, nrows=int(Xs.shape[0]), seconds=el, val_mse=val,
                       val_mse_zero=zero, gated=gated)


def eval_workload(ncol=262144, seed=0):
    """Evaluation set: 20-layer EnergyHydrology columns with the 65,536 x 15
    configuration's distributions (learned-guess evaluation configuration)."""
    return WL.learned_eval_c3(ncol=ncol, seed=seed)


def training_workload(ncol=65536, seed=0):
    return WL.energy_hydrology_c1(ncol=ncol, nlayers=LAYERS, seed=200 + seed)

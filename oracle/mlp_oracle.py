"""ORACLE — test infrastructure only.

FP64 NumPy restatement of the learned-guess network's forward pass and the
gradient of its training loss (mean over rows of the summed squared
standardised error), with inputs and weights rounded to BF16 as the GPU
kernels use them. The GPU gradients are checked against this.
"""
import numpy as np
from math import erf, sqrt, pi

N_IN, N_IN_PAD, N_H, N_OUT = 67, 80, 64, 40


def bf16(a):
    """Round float32 values to the nearest bfloat16 (ties to even)."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(erf)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / sqrt(2.0))) + x * np.exp(-0.5 * x * x) / sqrt(2.0 * pi)


def unpack(params):
    p = np.asarray(params, np.float64)
    o = 0
    W1 = p[o:o + N_IN_PAD * N_H].reshape(N_IN_PAD, N_H); o += N_IN_PAD * N_H
    b1 = p[o:o + N_H]; o += N_H
    W2 = p[o:o + N_H * N_H].reshape(N_H, N_H); o += N_H * N_H
    b2 = p[o:o + N_H]; o += N_H
    W3 = p[o:o + N_H * N_OUT].reshape(N_H, N_OUT); o += N_H * N_OUT
    b3 = p[o:o + N_OUT]
    return W1, b1, W2, b2, W3, b3


def loss_and_grad(params, norm, X, Y):
    in_mean, in_std, out_mean, out_std = norm
    W1, b1, W2, b2, W3, b3 = unpack(params)
    W1, W2, W3 = bf16(W1), bf16(W2), bf16(W3)
    istd = np.where(in_std > 1e-20, 1.0 / in_std, 0.0)
    Xs = np.zeros((X.shape[0], N_IN_PAD))
    Xs[:, :N_IN] = (X.astype(np.float64) - in_mean) * istd
    Xs = bf16(Xs)
    T = (Y.astype(np.float64) - out_mean) / out_std
    A1 = Xs @ W1 + b1
    H1 = gelu(A1)
    A2 = H1 @ W2 + b2
    H2 = gelu(A2)
    Yp = H2 @ W3 + b3
    E = Yp - T
    n = X.shape[0]
    loss = float(np.sum(E * E))
    dY = 2.0 * E / n
    gW3 = H2.T @ dY
    gb3 = dY.sum(0)
    dA2 = (dY @ W3.T) * gelu_grad(A2)
    gW2 = H1.T @ dA2
    gb2 = dA2.sum(0)
    dA1 = (dA2 @ W2.T) * gelu_grad(A1)
    gW1 = Xs.T @ dA1
    gb1 = dA1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g, Yp * out_std + out_mean

"""NumPy reference of the learned-guess conv net (test infrastructure).

FP64 arithmetic with the operands of every matrix product rounded to BF16 exactly as the
GPU kernels round them (round to nearest even), so that the GPU forward pass and gradients
can be compared against it at accumulation-order tolerance.
"""
import numpy as np
from scipy.special import erf

from qpad_gb300.learned import layout


def bf16(a):
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).astype(np.float64)


def _gelu(x):
    return 0.5 * x * (1.0 + erf(x / np.sqrt(2.0)))


def _gelu_grad(x):
    return 0.5 * (1.0 + erf(x / np.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / np.sqrt(2.0 * np.pi)


def _im2col(X, nr, K):
    C, N = X.shape
    cols = np.zeros((C * K, N))
    n = np.arange(N)
    x = n % nr
    for ci in range(C):
        for tap in range(K):
            xs = x + tap - K // 2
            ok = (xs >= 0) & (xs < nr)
            cols[ci * K + tap, ok] = X[ci, (n - x + xs)[ok]]
    return cols


def _col2im(dcols, C, nr, K):
    N = dcols.shape[1]
    dX = np.zeros((C, N))
    n = np.arange(N)
    x = n % nr
    for ci in range(C):
        for tap in range(K):
            xo = x - tap + K // 2
            ok = (xo >= 0) & (xo < nr)
            dX[ci, ok] += dcols[ci * K + tap, (n - x + xo)[ok]]
    return dX


def _unflat(p, cin, cout, width, layers, K):
    lay, _ = layout(cin, cout, width, layers, K)
    return [(p[wo:wo + np.prod(sh)].reshape(sh[0], sh[1] * sh[2]).astype(np.float64),
             p[bo:bo + sh[0]].astype(np.float64)) for wo, sh, bo in lay]


def forward(p, x, cin, cout, width, layers, K):
    ns, _, nr = x.shape
    X = np.transpose(x, (1, 0, 2)).reshape(cin, ns * nr).astype(np.float64)
    cache = []
    for l, (W, b) in enumerate(_unflat(p, cin, cout, width, layers, K)):
        cols = _im2col(X, nr, K)
        pre = bf16(W) @ bf16(cols) + b[:, None]
        cache.append((X, cols, pre))
        X = _gelu(pre) if l < layers - 1 else pre
        if l < layers - 1:
            X = X.astype(np.float32).astype(np.float64)   # activations are stored in FP32
    y = np.transpose(X.reshape(cout, ns, nr), (1, 0, 2))
    return y, cache


def loss_grad(p, x, t, cin, cout, width, layers, K):
    ns, _, nr = x.shape
    y, cache = forward(p, x, cin, cout, width, layers, K)
    d = y - t
    loss = float(np.mean(d * d))
    dY = (2.0 / d.size) * np.transpose(d, (1, 0, 2)).reshape(cout, ns * nr)
    dY = dY.astype(np.float32).astype(np.float64)
    params = _unflat(p, cin, cout, width, layers, K)
    lay, n = layout(cin, cout, width, layers, K)
    g = np.zeros(n)
    dcur = dY
    for l in range(layers - 1, -1, -1):
        X, cols, pre = cache[l]
        W, _ = params[l]
        if l < layers - 1:
            dcur = (dcur * _gelu_grad(pre)).astype(np.float32).astype(np.float64)
        wo, sh, bo = lay[l]
        g[bo:bo + sh[0]] = dcur.sum(axis=1)
        g[wo:wo + np.prod(sh)] = (bf16(dcur) @ bf16(cols).T).ravel()
        if l > 0:
            dcols = bf16(W).T @ bf16(dcur)
            dcur = _col2im(dcols.astype(np.float32).astype(np.float64), sh[1], nr, K)
    return loss, g

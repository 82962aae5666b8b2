"""Test infrastructure: an FP64 numpy restatement of the cost model's MLP
(the library's spmm_mlp_forward / spmm_mlp_backward), used only to check the
CUDA kernels.

Same parameter layout as the library: mu[in], sigma[in], then per layer
W[fan_out x fan_in] (row-major) and b[fan_out]; hidden layers use the exact
GELU x * Phi(x); loss = sum(mask (y - t)^2) / sum(mask); the gradient of mu
and sigma is zero (they are not trained).
"""
import math

import numpy as np

try:
    from scipy.special import erf as _erf
except ImportError:  # pragma: no cover
    _erf = np.vectorize(math.erf)


def _unpack(dims, p):
    n_in = dims[0]
    mu, sigma = p[:n_in], p[n_in:2 * n_in]
    off = 2 * n_in
    layers = []
    for l in range(len(dims) - 1):
        fi, fo = dims[l], dims[l + 1]
        W = p[off:off + fo * fi].reshape(fo, fi)
        off += fo * fi
        b = p[off:off + fo]
        off += fo
        layers.append((W, b))
    assert off == p.size, (off, p.size)
    return mu, sigma, layers


def dims_of(n_in, hidden, layers, n_out):
    return [n_in] + [hidden] * layers + [n_out]


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2 * math.pi)


def forward(dims, params, X, keep=False):
    p = np.asarray(params, np.float64)
    mu, sigma, layers = _unpack(dims, p)
    a = (np.asarray(X, np.float64) - mu) / sigma
    acts, zs = [a], []
    for l, (W, b) in enumerate(layers):
        z = a @ W.T + b
        zs.append(z)
        a = gelu(z) if l < len(layers) - 1 else z
        acts.append(a)
    return (a, acts, zs) if keep else a


def loss_grad(dims, params, X, T, mask):
    p = np.asarray(params, np.float64)
    Y, acts, zs = forward(dims, p, X, keep=True)
    T = np.asarray(T, np.float64)
    M = np.asarray(mask, np.float64)
    cnt = M.sum() if M.sum() > 0 else 1.0
    d = (Y - T) * M
    loss = float((M * (Y - T) ** 2).sum() / cnt)
    dz = 2.0 * d / cnt
    mu, sigma, layers = _unpack(dims, p)
    grads = []
    for l in range(len(layers) - 1, -1, -1):
        W, _ = layers[l]
        gW = dz.T @ acts[l]
        gb = dz.sum(axis=0)
        grads.append((gW, gb))
        if l > 0:
            dz = (dz @ W) * gelu_grad(zs[l - 1])
    grads.reverse()
    g = [np.zeros(2 * dims[0])]
    for gW, gb in grads:
        g += [gW.ravel(), gb]
    return loss, np.concatenate(g)

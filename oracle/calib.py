"""ORACLE — test infrastructure only.  FP64 restatement of the mixture NLL and
its gradient (no reference counterpart: ProCESS has no calibration path), in
numpy, written from the model definition independently of the CUDA adjoint:
the gradient is obtained by differentiating the per-site log-sum-exp term by
term, and checked against central finite differences."""
from __future__ import annotations

import numpy as np


def _softmax(x, axis=-1):
    e = np.exp(x - x.max(axis=axis, keepdims=True))
    return e / e.sum(axis=axis, keepdims=True)


def nll(params, alt, depth, cls, sig, L, phi, K, J):
    """NLL of one replicate (FP64)."""
    lr, th, rho = params[:K], params[K:K + K * J].reshape(K, J), params[K + K * J]
    sig = sig / sig.sum(axis=1, keepdims=True)
    w = _softmax(th, axis=1)
    M = w @ sig                                     # K x C
    logw = lr + np.log(L)
    logpi = logw[:, None] + np.log(M) - np.logaddexp.reduce(logw)
    purity = 1.0 / (1.0 + np.exp(-rho))
    v = purity * phi / 2
    a = alt.astype(np.float64)[:, None]
    d = depth.astype(np.float64)[:, None]
    t = logpi[:, cls].T + a * np.log(v)[None, :] + (d - a) * np.log1p(-v)[None, :]
    return -np.logaddexp.reduce(t, axis=1).sum()


def nll_grad(params, alt, depth, cls, sig, L, phi, K, J):
    """NLL and its analytic gradient (FP64)."""
    params = np.asarray(params, dtype=np.float64)
    lr, th, rho = params[:K], params[K:K + K * J].reshape(K, J), params[K + K * J]
    sig = sig / sig.sum(axis=1, keepdims=True)
    w = _softmax(th, axis=1)                        # K x J
    M = w @ sig                                     # K x C
    rates = np.exp(lr) * L
    Z = rates.sum()
    logpi = np.log(rates / Z)[:, None] + np.log(M)
    purity = 1.0 / (1.0 + np.exp(-rho))
    v = purity * phi / 2
    a = alt.astype(np.float64)[:, None]
    d = depth.astype(np.float64)[:, None]
    t = logpi[:, cls].T + a * np.log(v)[None, :] + (d - a) * np.log1p(-v)[None, :]   # n x K
    ll = np.logaddexp.reduce(t, axis=1)
    gam = np.exp(t - ll[:, None])                   # responsibilities
    n = len(alt)
    g = np.zeros_like(params)
    # log pi_k(c) = lr_k + log L_k - log Z + log M_k(c)
    Gk = gam.sum(axis=0)
    g[:K] = -(Gk - n * rates / Z)
    # d log M_k(c) / d theta_kj = w_kj (S_j(c) - M_k(c)) / M_k(c)
    for k in range(K):
        ratio = sig[:, cls] / M[k, cls][None, :]     # J x n
        g[K + k * J:K + (k + 1) * J] = -w[k] * ((ratio * gam[:, k][None, :]).sum(axis=1) - Gk[k])
    # d t_ik / d rho = (a/v_k - (d-a)/(1-v_k)) v_k (1 - purity)
    dt = (a / v[None, :] - (d - a) / (1 - v[None, :])) * v[None, :] * (1 - purity)
    g[K + K * J] = -(gam * dt).sum()
    return -ll.sum(), g


def finite_diff(params, h, *args):
    """Central finite differences of nll (FP64)."""
    params = np.asarray(params, dtype=np.float64)
    out = np.zeros_like(params)
    for q in range(len(params)):
        e = np.zeros_like(params)
        e[q] = h
        out[q] = (nll(params + e, *args) - nll(params - e, *args)) / (2 * h)
    return out

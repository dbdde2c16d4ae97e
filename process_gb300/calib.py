"""Calibration of epoch rates, exposures and purity from alt/depth tables.

The expected-VAF binomial-mixture negative log-likelihood and its adjoint run
in the CUDA library (``pg_calib_*`` in include/process_gb300.h).  This module
holds the host-side batch, a thin ``torch.autograd.Function`` used for
gradient checks and calibration loops written in torch, and the synthetic
tables of the calibration workloads.

Parameters of a replicate (P = K + K*J + 1): log rates ``lr_k``, exposure
logits ``theta_kj`` (softmax over j per epoch) and the purity logit ``rho``.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _lib
from ._lib import check, lib, ptr


def _bind():
    L = lib()
    P = C.c_void_p
    protos = {
        "pg_calib_create": (C.c_int, [C.c_uint32, C.POINTER(C.c_uint64), C.POINTER(C.c_int32),
                                      C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_uint32, C.c_uint32,
                                      C.c_uint32, C.POINTER(C.c_double), C.POINTER(C.c_double),
                                      C.POINTER(C.c_double), C.POINTER(P)]),
        "pg_calib_destroy": (C.c_int, [P]),
        "pg_calib_num_params": (C.c_int, [P, C.POINTER(C.c_uint32)]),
        "pg_calib_set_stream": (C.c_int, [P, P]),
        "pg_calib_nll_grad": (C.c_int, [P, P, P, P]),
        "pg_calib_nll_grad_one": (C.c_int, [P, C.c_uint32, P, P, P]),
        "pg_calib_adam": (C.c_int, [P, P, C.c_uint32, C.c_float, C.c_float, C.c_float, C.c_float, P]),
    }
    for name, (res, args) in protos.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def n_params(K: int, J: int) -> int:
    return K + K * J + 1


def pack_params(lr, theta, rho) -> np.ndarray:
    """[lr_0..K-1, theta_00..theta_K-1,J-1, rho] for one replicate."""
    return np.concatenate([np.ravel(lr), np.ravel(theta), [rho]]).astype(np.float64)


def unpack_params(p, K: int, J: int):
    p = np.asarray(p)
    return p[..., :K], p[..., K:K + K * J].reshape(p.shape[:-1] + (K, J)), p[..., K + K * J]


class CalibBatch:
    """Device-resident alt/depth/class tables of ``n_rep`` replicates."""

    def __init__(self, site_off, alt, depth, cls, signatures, epoch_weight, phi):
        self.L = _bind()
        site_off = np.ascontiguousarray(site_off, dtype=np.uint64)
        alt = np.ascontiguousarray(alt, dtype=np.int32)
        depth = np.ascontiguousarray(depth, dtype=np.int32)
        cls = np.ascontiguousarray(cls, dtype=np.int32)
        sig = np.ascontiguousarray(signatures, dtype=np.float64)
        ew = np.ascontiguousarray(epoch_weight, dtype=np.float64)
        ph = np.ascontiguousarray(phi, dtype=np.float64)
        self.n_rep = len(site_off) - 1
        self.J, self.C = sig.shape
        self.K = ew.shape[1]
        self.P = n_params(self.K, self.J)
        self.n_sites = int(site_off[-1])
        h = C.c_void_p()
        check(self.L.pg_calib_create(self.n_rep, ptr(site_off, C.c_uint64), ptr(alt, C.c_int32),
                                     ptr(depth, C.c_int32), ptr(cls, C.c_int32), self.K, self.J, self.C,
                                     ptr(sig, C.c_double), ptr(ew, C.c_double), ptr(ph, C.c_double), C.byref(h)))
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _lib._LIB is not None:
            self.L.pg_calib_destroy(h)
            self._h = None

    def nll_grad(self, params):
        """NLL (n_rep,) and gradient (n_rep, P) for a CUDA float32 tensor (n_rep, P)."""
        import torch
        params = params.detach().to(dtype=torch.float32).contiguous()
        nll = torch.empty(self.n_rep, dtype=torch.float32, device=params.device)
        grad = torch.empty_like(params)
        with self._on_stream(params, nll, grad):
            check(self.L.pg_calib_nll_grad(self._h, C.c_void_p(params.data_ptr()), C.c_void_p(nll.data_ptr()),
                                           C.c_void_p(grad.data_ptr())))
        return nll, grad

    def nll_grad_one(self, rep: int, params):
        """Per-instance path: replicate ``rep`` only, writing rows ``rep`` of nll/grad."""
        import torch
        nll = torch.zeros(self.n_rep, dtype=torch.float32, device=params.device)
        grad = torch.zeros_like(params)
        with self._on_stream(params, nll, grad):
            check(self.L.pg_calib_nll_grad_one(self._h, rep, C.c_void_p(params.data_ptr()),
                                               C.c_void_p(nll.data_ptr()), C.c_void_p(grad.data_ptr())))
        return nll, grad

    def adam(self, params, steps: int, lr: float = 0.05, beta1: float = 0.9, beta2: float = 0.999,
             eps: float = 1e-8):
        """``steps`` Adam steps on every replicate, in place, as one CUDA graph."""
        import torch
        assert params.dtype == torch.float32 and params.is_contiguous() and params.is_cuda
        nll = torch.empty(self.n_rep, dtype=torch.float32, device=params.device)
        with self._on_stream(params, nll):
            check(self.L.pg_calib_adam(self._h, C.c_void_p(params.data_ptr()), steps, lr, beta1, beta2, eps,
                                       C.c_void_p(nll.data_ptr())))
        return nll

    @property
    def stream(self):
        """The torch stream the handle's kernels run on (created on first use)."""
        import torch
        if getattr(self, "_stream", None) is None:
            self._stream = torch.cuda.Stream()
            check(self.L.pg_calib_set_stream(self._h, C.c_void_p(self._stream.cuda_stream)))
        return self._stream

    def _on_stream(self, *tensors):
        """Orders the call after the caller's stream and the caller's stream after the call."""
        import contextlib

        import torch

        @contextlib.contextmanager
        def ctx():
            cur = torch.cuda.current_stream()
            s = self.stream
            s.wait_stream(cur)
            for t in tensors:
                t.record_stream(s)
            yield
            cur.wait_stream(s)

        return ctx()


def _autograd():
    import torch

    class MixtureNLL(torch.autograd.Function):
        """Sum over replicates of the mixture NLL; backward uses the CUDA adjoint."""

        @staticmethod
        def forward(ctx, params, batch: CalibBatch):
            nll, grad = batch.nll_grad(params)
            ctx.save_for_backward(grad)
            return nll.sum()

        @staticmethod
        def backward(ctx, g):
            (grad,) = ctx.saved_tensors
            return g * grad, None

    return MixtureNLL


def mixture_nll(params, batch: CalibBatch):
    """Differentiable (torch) sum of the replicates' NLLs."""
    return _autograd().apply(params, batch)


# ---------------------------------------------------------------- synthetic tables
@dataclass
class CalibData:
    site_off: np.ndarray
    alt: np.ndarray
    depth: np.ndarray
    cls: np.ndarray
    signatures: np.ndarray     # J x C
    epoch_weight: np.ndarray   # R x K
    phi: np.ndarray            # R x K
    true_params: np.ndarray    # R x P

    @property
    def n_rep(self):
        return len(self.site_off) - 1


def synthetic(n_rep: int, n_sites: int, depth_means, seed: int, K: int = 4, J: int = 3, C: int = 96) -> CalibData:
    """Sites drawn from the model itself: epoch ~ pi, class ~ M_k, depth ~
    Poisson(mean of the replicate), alt ~ Binomial(depth, v_k).  Per replicate:
    Dirichlet(1) exposures over J shared Dirichlet(0.5) signatures, log-uniform
    epoch rates, purity U(0.5, 0.95).  Sites with depth 0 are dropped."""
    rng = np.random.default_rng(seed)
    sig = rng.dirichlet(np.full(C, 0.5), size=J)
    depth_means = np.broadcast_to(np.asarray(depth_means, dtype=np.float64), (n_rep,))
    L = np.tile(np.arange(1, K + 1, dtype=np.float64), (n_rep, 1))
    phi = np.tile(np.array([1.0, 0.6, 0.35, 0.2][:K] + [0.1] * max(0, K - 4)), (n_rep, 1))
    true = np.zeros((n_rep, n_params(K, J)))
    offs, alts, deps, clss = [0], [], [], []
    for r in range(n_rep):
        lrate = np.log(rng.uniform(0.5, 2.0, K))
        w = rng.dirichlet(np.ones(J), size=K)
        theta = np.log(w)
        purity = rng.uniform(0.5, 0.95)
        rho = np.log(purity / (1 - purity))
        true[r] = pack_params(lrate, theta, rho)
        pi_k = np.exp(lrate) * L[r]
        pi_k /= pi_k.sum()
        k = rng.choice(K, size=n_sites, p=pi_k)
        M = w @ sig
        u = rng.random(n_sites)
        cls = (M[k].cumsum(axis=1) < u[:, None]).sum(axis=1).clip(0, C - 1)
        d = rng.poisson(depth_means[r], n_sites)
        v = purity * phi[r, k] / 2
        a = rng.binomial(d, v)
        keep = d > 0
        alts.append(a[keep]); deps.append(d[keep]); clss.append(cls[keep])
        offs.append(offs[-1] + int(keep.sum()))
    return CalibData(np.array(offs, dtype=np.uint64), np.concatenate(alts).astype(np.int32),
                     np.concatenate(deps).astype(np.int32), np.concatenate(clss).astype(np.int32), sig, L, phi,
                     true)


def batch_of(d: CalibData) -> CalibBatch:
    return CalibBatch(d.site_off, d.alt, d.depth, d.cls, d.signatures, d.epoch_weight, d.phi)

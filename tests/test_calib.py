"""Calibration NLL and adjoint: FP64 oracle against finite differences (CPU);
the FP32 CUDA adjoint against the FP64 gradient and finite differences, the
batched against the per-instance path, and batched Adam recovery (GPU)."""
import numpy as np
import pytest


def _rep(d, r, K=4, J=3, n=None):
    s, e = int(d.site_off[r]), int(d.site_off[r + 1])
    if n is not None:
        e = min(e, s + n)
    return (d.alt[s:e], d.depth[s:e], d.cls[s:e], d.signatures, d.epoch_weight[r], d.phi[r], K, J)


def test_oracle_gradient_matches_finite_differences():
    import oracle.calib as oc
    from process_gb300 import calib
    d = calib.synthetic(1, 5000, 100, seed=1)
    p = d.true_params[0] + np.random.default_rng(2).normal(0, 0.3, d.true_params.shape[1])
    f, g = oc.nll_grad(p, *_rep(d, 0))
    fd = oc.finite_diff(p, 1e-5, *_rep(d, 0))
    assert np.isclose(f, oc.nll(p, *_rep(d, 0)), rtol=1e-12)
    assert np.linalg.norm(g - fd) / np.linalg.norm(fd) < 1e-6


def test_synthetic_tables_shape():
    from process_gb300 import calib
    d = calib.synthetic(3, 1000, [30, 100, 200], seed=5)
    assert d.n_rep == 3 and d.site_off[-1] == len(d.alt)
    assert np.all(d.alt <= d.depth) and np.all(d.depth > 0)
    assert d.true_params.shape == (3, calib.n_params(4, 3))


@pytest.mark.gpu
def test_adjoint_matches_fp64_gradient_2e5_sites(gpu_lib):
    """2e5 sites, depth ~ Poisson(100), K=4, 3 exposures per epoch: FP32 adjoint
    against the FP64 gradient and FP64 central differences (h = 1e-5),
    relative error < 1e-4."""
    import torch

    import oracle.calib as oc
    from process_gb300 import calib
    d = calib.synthetic(1, 200_000, 100, seed=4)
    b = calib.batch_of(d)
    rng = np.random.default_rng(7)
    for trial in range(3):
        p = d.true_params + rng.normal(0, 0.4, d.true_params.shape)
        pt = torch.tensor(p, dtype=torch.float32, device="cuda")
        nll, grad = b.nll_grad(pt)
        torch.cuda.synchronize()
        # the oracle evaluates at the FP32-rounded parameters the kernel saw
        p32 = pt.double().cpu().numpy()[0]
        f, g = oc.nll_grad(p32, *_rep(d, 0))
        gg = grad.double().cpu().numpy()[0]
        assert abs(float(nll[0]) - f) / abs(f) < 1e-5
        assert np.linalg.norm(gg - g) / np.linalg.norm(g) < 1e-4
        if trial == 0:
            fd = oc.finite_diff(p32, 1e-5, *_rep(d, 0))
            assert np.linalg.norm(gg - fd) / np.linalg.norm(fd) < 1e-4


@pytest.mark.gpu
def test_adjoint_replicates_off_the_four_site_grid(gpu_lib):
    """Replicates of 10,001 sites: every chunk but the first starts and ends
    off a multiple of four sites, so the kernel's site-by-site head and tail
    run beside its four-site loads; each replicate against the FP64 gradient."""
    import torch

    import oracle.calib as oc
    from process_gb300 import calib
    d = calib.synthetic(3, 10_001, [40, 90, 160], seed=12)
    assert d.site_off[1] % 4 != 0
    b = calib.batch_of(d)
    p = torch.tensor(d.true_params + 0.3, dtype=torch.float32, device="cuda")
    nll, grad = b.nll_grad(p)
    torch.cuda.synchronize()
    p32 = p.double().cpu().numpy()
    for r in range(d.n_rep):
        f, g = oc.nll_grad(p32[r], *_rep(d, r))
        gg = grad.double().cpu().numpy()[r]
        assert abs(float(nll[r]) - f) / abs(f) < 1e-5
        assert np.linalg.norm(gg - g) / np.linalg.norm(g) < 1e-4


@pytest.mark.gpu
def test_batched_equals_per_instance_and_autograd(gpu_lib):
    import torch

    from process_gb300 import calib
    d = calib.synthetic(6, 30_000, [30, 60, 90, 120, 150, 200], seed=9)
    b = calib.batch_of(d)
    p = torch.tensor(d.true_params + 0.2, dtype=torch.float32, device="cuda")
    nll, grad = b.nll_grad(p)
    for r in range(d.n_rep):
        n1, g1 = b.nll_grad_one(r, p)
        assert torch.equal(n1[r], nll[r]) and torch.equal(g1[r], grad[r])
    x = p.clone().requires_grad_(True)
    loss = calib.mixture_nll(x, b)
    loss.backward()
    assert torch.allclose(loss, nll.sum()) and torch.equal(x.grad, grad)


@pytest.mark.gpu
def test_batched_adam_recovers_exposures(gpu_lib):
    """200 Adam steps on the device under one CUDA graph: recovered exposures
    within L1 0.05 of the seeded truth per epoch, purity within 0.02."""
    import torch

    from process_gb300 import calib
    d = calib.synthetic(8, 100_000, np.linspace(30, 200, 8), seed=11)
    b = calib.batch_of(d)
    p = torch.zeros((d.n_rep, b.P), dtype=torch.float32, device="cuda")
    b.adam(p, 200, lr=0.05)
    torch.cuda.synchronize()
    K, J = 4, 3
    _, th, rho = calib.unpack_params(p.double().cpu().numpy(), K, J)
    _, tht, rhot = calib.unpack_params(d.true_params, K, J)
    w = np.exp(th) / np.exp(th).sum(-1, keepdims=True)
    wt = np.exp(tht) / np.exp(tht).sum(-1, keepdims=True)
    l1 = np.abs(w - wt).sum(-1)
    assert l1.mean() < 0.05 and l1.max() < 0.12
    pur, purt = 1 / (1 + np.exp(-rho)), 1 / (1 + np.exp(-rhot))
    assert np.abs(pur - purt).max() < 0.02


@pytest.mark.gpu
@pytest.mark.parametrize("K,J,C", [(2, 6, 40), (5, 1, 96), (8, 8, 128), (1, 4, 7), (3, 5, 96)])
def test_adjoint_other_shapes(gpu_lib, K, J, C):
    """Every (epochs, signatures) shape has its own site kernel: the FP32
    adjoint against the FP64 gradient, relative error < 1e-4, over two
    replicates of different depth."""
    import torch

    import oracle.calib as oc
    from process_gb300 import calib
    d = calib.synthetic(2, 40_000, [60, 150], seed=20 + K * 8 + J, K=K, J=J, C=C)
    b = calib.batch_of(d)
    p = d.true_params + np.random.default_rng(K * 10 + J).normal(0, 0.3, d.true_params.shape)
    pt = torch.tensor(p, dtype=torch.float32, device="cuda")
    nll, grad = b.nll_grad(pt)
    torch.cuda.synchronize()
    p32 = pt.double().cpu().numpy()
    for r in range(2):
        f, g = oc.nll_grad(p32[r], *_rep(d, r, K=K, J=J))
        gg = grad.double().cpu().numpy()[r]
        assert abs(float(nll[r]) - f) / abs(f) < 1e-5
        assert np.linalg.norm(gg - g) / np.linalg.norm(g) < 1e-4

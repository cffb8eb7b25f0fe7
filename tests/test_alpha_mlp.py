"""The learned-alpha network: the numpy reference gradient against finite
differences (CPU), and the GPU training kernels' gradient against the numpy
reference (GPU)."""
import numpy as np
import pytest

from oracle import mlp_ref


def _records(n, seed=0):
    rng = np.random.default_rng(seed)
    x = rng.uniform(-1, 1, (n, 27))
    x /= np.abs(x).max(axis=1, keepdims=True)
    lam = rng.uniform(1e-3, 0.1, n)
    t = 0.3 * x[:, 0] ** 3 - 0.1 * x[:, 5] + 0.05 * np.sin(3 * x[:, 9])
    return np.concatenate([x, lam[:, None], t[:, None]], axis=1)


def test_reference_gradient_matches_finite_differences():
    w = mlp_ref.init(1)
    rec = _records(64)
    loss, g = mlp_ref.loss_and_grad(w, rec)
    rng = np.random.default_rng(2)
    for k in rng.choice(mlp_ref.NPARAM, 40, replace=False):
        e = np.zeros_like(w)
        e[k] = 1e-6
        fd = (mlp_ref.loss_and_grad(w + e, rec)[0] - mlp_ref.loss_and_grad(w - e, rec)[0]) / 2e-6
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(g[k])) + 1e-9, k
    assert mlp_ref.NPARAM == 6017


@pytest.mark.gpu
def test_gpu_gradient_matches_reference(pkg, built_lib):
    ctx = pkg.capi.Context(0)
    w = mlp_ref.init(3).astype(np.float32)
    rec = _records(3000, seed=4).astype(np.float32)
    g_gpu, loss_gpu = ctx.alpha_mlp_grad(w, rec)
    loss_ref, g_ref = mlp_ref.loss_and_grad(w.astype(np.float64), rec.astype(np.float64))
    assert abs(loss_gpu - loss_ref) <= 1e-5 * loss_ref
    err = np.abs(g_gpu - g_ref) / (np.abs(g_ref).max() + 1e-30)
    assert err.max() <= 1e-4, err.max()
    ctx.close()


@pytest.mark.gpu
def test_gpu_training_reduces_loss(pkg, built_lib):
    ctx = pkg.capi.Context(0)
    rec = _records(20000, seed=5).astype(np.float32)
    w0 = mlp_ref.init(6).astype(np.float32)
    w1, hist = ctx.alpha_mlp_train(rec, w0, epochs=6, batch=1000, lr=3e-3, seed=1)
    assert np.isfinite(hist).all() and hist[-1] < 0.2 * hist[0], hist
    l0 = mlp_ref.loss_and_grad(w0.astype(np.float64), rec)[0]
    l1 = mlp_ref.loss_and_grad(w1.astype(np.float64), rec)[0]
    assert l1 < 0.2 * l0
    ctx.close()

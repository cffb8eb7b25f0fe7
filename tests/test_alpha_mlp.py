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
    assert np.isfinite(hist).all() and np.all(np.diff(hist) < 0) and hist[-1] < 0.5 * hist[0], hist
    l0 = mlp_ref.loss_and_grad(w0.astype(np.float64), rec)[0]
    l1 = mlp_ref.loss_and_grad(w1.astype(np.float64), rec)[0]
    assert l1 < 0.2 * l0
    ctx.close()


def _bf16(a):
    """Round float32 values to BF16 (nearest even), returned as float32."""
    u = np.ascontiguousarray(a, np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32)


@pytest.mark.gpu
@pytest.mark.parametrize("n", [128, 1000, 20000])
def test_gpu_tensor_core_inference(pkg, built_lib, n):
    """tcgen05 inference (BF16 operands, FP32 accumulation in tensor memory)
    against a numpy model of the same roundings, and against FP64."""
    ctx = pkg.capi.Context(0)
    rng = np.random.default_rng(11)
    p = mlp_ref.unpack(mlp_ref.init(7))
    for b in ("b1", "b2", "b3"):
        p[b] = rng.normal(0, 0.3, p[b].shape)
    w = mlp_ref.pack(p).astype(np.float32)
    x = rng.uniform(-1, 1, (n, 27))
    x /= np.abs(x).max(axis=1, keepdims=True)
    x = x.astype(np.float32)
    out, status = ctx.alpha_mlp_infer(w, x)
    ctx.close()
    assert status == 0
    q = mlp_ref.unpack(w.astype(np.float64))
    g = lambda z: mlp_ref.gelu(z)[0]
    h1 = _bf16(g(_bf16(x).astype(np.float64) @ _bf16(q["W1"]) + q["b1"]))
    ref = g(h1.astype(np.float64) @ _bf16(q["W2"]) + q["b2"]) @ q["w3"] + q["b3"][0]
    exact = mlp_ref.forward(w.astype(np.float64), x.astype(np.float64))[0]
    scale = np.sqrt(np.mean(exact ** 2))
    assert np.max(np.abs(out - ref)) <= 2e-2 * scale, np.max(np.abs(out - ref)) / scale
    assert np.sqrt(np.mean((out - exact) ** 2)) <= 2e-2 * scale

"""The warm-start MLP's GPU kernels (BF16 tensor-core GEMMs, FP32 accumulation,
Adam) against the CPU restatement in oracle/mlp_oracle.py.

The GPU rounds activations and their gradients to BF16 (8-bit mantissa); the
oracle works in FP64 on the same BF16-rounded weights and inputs.  Tolerances,
written per check: loss to 1e-2 relative, every parameter tensor's gradient
to 5e-2 relative in the 2-norm with cosine similarity above 0.998."""
import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d
from gpueularsolver2d_gb300._lib import E2DError

pytestmark = pytest.mark.gpu


def test_gradient_matches_cpu_oracle(lib, oracle):
    import mlp_oracle
    B, L = 2048, 3
    net = e2d.MLP(nhidden=L, batch=B, seed=11)
    rng = np.random.default_rng(5)
    x = np.zeros((B, 32), np.float32)
    x[:, :22] = rng.normal(size=(B, 22)).astype(np.float32)
    t = rng.normal(size=(B, 4)).astype(np.float32) * 0.3
    loss, g = net.gradient(x, t)
    p = net.params()
    loss_ref, g_ref = mlp_oracle.loss_and_grad(p, x, t, L)
    assert abs(loss - loss_ref) / loss_ref < 1e-2
    off = 0
    for l in range(L + 1):
        rows = 4 if l == L else 256
        cols = 32 if l == 0 else 256
        for size in (rows * cols, rows):
            a, b = g[off:off + size].astype(np.float64), g_ref[off:off + size]
            off += size
            if l == 0 and size == rows * cols:  # padding inputs have zero gradient
                a = a.reshape(rows, cols)[:, :22].ravel()
                b = b.reshape(rows, cols)[:, :22].ravel()
            rel = np.linalg.norm(a - b) / np.linalg.norm(b)
            cos = a @ b / (np.linalg.norm(a) * np.linalg.norm(b))
            assert rel < 5e-2 and cos > 0.998, (l, size, rel, cos)
    assert off == len(g)


def test_training_reduces_loss_and_forward_agrees(lib):
    B = 4096
    net = e2d.MLP(nhidden=3, batch=B, seed=2, lr=2e-3)
    rng = np.random.default_rng(0)
    n = 40000
    x = np.zeros((n, 32), np.float32)
    x[:, :22] = rng.uniform(-1, 1, size=(n, 22)).astype(np.float32)
    t = np.stack([np.sin(2 * x[:, 0]) * x[:, 1], np.cos(x[:, 2] + x[:, 3]), x[:, 4] ** 2 - 0.3,
                  0.5 * np.tanh(3 * x[:, 5])], axis=1).astype(np.float32)
    net.set_data(x, t)
    loss = net.train(400)
    assert np.all(np.isfinite(loss))
    assert loss[-20:].mean() < 0.1 * loss[:5].mean(), (loss[:5].mean(), loss[-20:].mean())
    y = net.forward(x[:5000])
    mse = float(np.mean((y - t[:5000]) ** 2))
    assert mse < 2.0 * loss[-20:].mean() + 1e-4


def test_adam_step_size_is_scheduled_on_device(lib):
    """e2d_mlp_set_lr changes the step size of the steps that follow: lr 0
    leaves every parameter as it was; Adam's first step moves each parameter
    by lr * |g| / (|g| + eps), i.e. by lr wherever the gradient is not tiny,
    and not at all where it is zero (the padding inputs of the first layer)."""
    B = 2048
    rng = np.random.default_rng(1)
    n = 8192
    x = np.zeros((n, 32), np.float32)
    x[:, :22] = rng.uniform(-1, 1, size=(n, 22)).astype(np.float32)
    t = rng.normal(size=(n, 4)).astype(np.float32)
    net = e2d.MLP(nhidden=2, batch=B, seed=4, lr=1e-3)
    net.set_data(x, t)
    p0 = net.params()
    net.set_lr(0.0)
    net.train(3, record_loss=False)
    assert np.array_equal(net.params(), p0)
    with pytest.raises(E2DError):
        net.set_lr(-1.0)
    net2 = e2d.MLP(nhidden=2, batch=B, seed=4, lr=1.0)
    net2.set_data(x, t)
    q0 = net2.params()
    lr = 1e-3
    net2.set_lr(lr)
    net2.train(1, record_loss=False)
    d = np.abs(net2.params().astype(np.float64) - q0)
    w0 = d[:256 * 32].reshape(256, 32)
    assert np.all(w0[:, 22:] == 0.0)
    assert np.all(d <= lr * (1 + 1e-3) + 1e-6)
    moved = d[d > 0]
    assert np.median(np.abs(moved - lr)) < 1e-6, np.median(moved)


def test_warp_specialised_gemms_match_per_tile_gemms(lib):
    """The hidden-layer GEMMs of the persistent TMA / tcgen05 kernel (weights
    resident in shared memory, two accumulators in tensor memory) against the
    per-tile kernel (E2D_MLP_WS=0) on the same network and batch: forward
    outputs and every gradient agree to the accumulation order (bf16 storage
    of activations and gradients)."""
    import os
    B, L = 4096, 4
    rng = np.random.default_rng(9)
    x = np.zeros((B, 32), np.float32)
    x[:, :22] = rng.normal(size=(B, 22)).astype(np.float32)
    t = rng.normal(size=(B, 4)).astype(np.float32) * 0.3
    out = {}
    for mode in ("1", "0"):
        os.environ["E2D_MLP_WS"] = mode
        try:
            net = e2d.MLP(nhidden=L, batch=B, seed=4)
            loss, g = net.gradient(x, t)
            out[mode] = (net.forward(x), loss, g)
            net.close()
        finally:
            os.environ.pop("E2D_MLP_WS", None)
    (y1, l1, g1), (y0, l0, g0) = out["1"], out["0"]
    assert np.max(np.abs(y1 - y0)) <= 1e-2 * np.max(np.abs(y0)) + 1e-6
    assert abs(l1 - l0) <= 1e-3 * abs(l0)
    cos = float(g1 @ g0 / (np.linalg.norm(g1) * np.linalg.norm(g0)))
    assert cos > 0.9999 and np.linalg.norm(g1 - g0) < 2e-2 * np.linalg.norm(g0), cos

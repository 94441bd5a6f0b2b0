"""CPU restatement of the warm-start MLP's loss and gradient (TEST INFRASTRUCTURE
ONLY: the checker of the GPU training kernels; no reference counterpart).

Same network as gpueularsolver2d_gb300/csrc/mlp.cu: 32 inputs -> nhidden x 256
(GELU, tanh form) -> 4 outputs, MSE loss over the batch and the 4 outputs.
Parameters in the order W0, b0, ..., W_out, b_out with W[out][in].  The GPU
rounds weights, inputs, activations and their gradients to BF16 and
accumulates in FP32; this restatement works in FP64 on the BF16-rounded
weights and inputs, so the comparison bounds the effect of the BF16
intermediates.
"""
import math

import numpy as np

H, NIN, NOUT = 256, 32, 4


def bf16_round(a: np.ndarray) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even)."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def unpack(p: np.ndarray, nhidden: int):
    Ws, bs, off = [], [], 0
    for l in range(nhidden + 1):
        rows = NOUT if l == nhidden else H
        cols = NIN if l == 0 else H
        Ws.append(p[off:off + rows * cols].reshape(rows, cols).astype(np.float64))
        off += rows * cols
        bs.append(p[off:off + rows].astype(np.float64))
        off += rows
    return Ws, bs


C0, C1 = math.sqrt(2.0 / math.pi), 0.044715


def gelu(z):
    """GELU, tanh form: z (1 + tanh(sqrt(2/pi) (z + 0.044715 z^3))) / 2."""
    return 0.5 * z * (1.0 + np.tanh(C0 * (z + C1 * z ** 3)))


def gelu_grad(z):
    t = np.tanh(C0 * (z + C1 * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * C0 * (1.0 + 3.0 * C1 * z * z)


def loss_and_grad(p: np.ndarray, x: np.ndarray, t: np.ndarray, nhidden: int):
    Ws, bs = unpack(p, nhidden)
    # the GPU multiplies hidden layers with BF16 weights; the output layer is FP32
    Wq = [bf16_round(W.astype(np.float32)).astype(np.float64) if l < nhidden else W for l, W in enumerate(Ws)]
    h = bf16_round(x.astype(np.float32)).astype(np.float64)
    zs, hs = [], [h]
    for l in range(nhidden):
        z = h @ Wq[l].T + bs[l]
        h = gelu(z)
        zs.append(z)
        hs.append(h)
    y = h @ Wq[nhidden].T + bs[nhidden]
    B = x.shape[0]
    d = y - t
    loss = float(np.sum(d * d) / (B * NOUT))
    dy = 2.0 * d / (B * NOUT)
    grads_W, grads_b = [None] * (nhidden + 1), [None] * (nhidden + 1)
    grads_W[nhidden] = dy.T @ hs[nhidden]
    grads_b[nhidden] = dy.sum(axis=0)
    dh = dy @ Wq[nhidden]
    for l in range(nhidden - 1, -1, -1):
        z = zs[l]
        dz = dh * gelu_grad(z)
        grads_W[l] = dz.T @ hs[l]
        grads_b[l] = dz.sum(axis=0)
        dh = dz @ Wq[l]
    flat = []
    for l in range(nhidden + 1):
        flat.append(grads_W[l].ravel())
        flat.append(grads_b[l].ravel())
    return loss, np.concatenate(flat)

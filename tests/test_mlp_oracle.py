"""The MLP oracle itself (CPU): its GELU derivative against a central
difference of its GELU, and its parameter gradient against central
differences of its loss on a small network.  The GPU kernels are checked
against this oracle in tests/test_mlp.py."""
import sys
from pathlib import Path

import numpy as np

sys.path.insert(0, str(Path(__file__).resolve().parents[1] / "oracle"))
import mlp_oracle as mo  # noqa: E402


def test_gelu_derivative():
    x = np.linspace(-8.0, 8.0, 4001)
    h = 1e-6
    fd = (mo.gelu(x + h) - mo.gelu(x - h)) / (2 * h)
    assert np.max(np.abs(fd - mo.gelu_grad(x))) < 1e-8
    # limits: gelu(x) -> x for large x, -> 0 for very negative x
    assert abs(mo.gelu(10.0) - 10.0) < 1e-12 and abs(mo.gelu(-10.0)) < 1e-12


def test_loss_gradient_against_finite_differences():
    rng = np.random.default_rng(2)
    L, B = 2, 16
    sizes = []
    for l in range(L + 1):
        rows = mo.NOUT if l == L else mo.H
        cols = mo.NIN if l == 0 else mo.H
        sizes += [rows * cols, rows]
    p = (rng.normal(size=sum(sizes)) * 0.05).astype(np.float32)
    x = np.zeros((B, mo.NIN), np.float32)
    x[:, :22] = rng.normal(size=(B, 22))
    t = rng.normal(size=(B, mo.NOUT)).astype(np.float32)
    # the oracle rounds hidden-layer weights to BF16; probe parameters whose
    # rounding does not move under the perturbation: output-layer weights
    # and biases (kept in FP32) and hidden biases
    loss, g = mo.loss_and_grad(p, x, t, L)
    offs = np.cumsum([0] + sizes)
    probes = list(range(offs[2 * L], offs[2 * L] + 8))  # output-layer weights
    probes += list(range(offs[1], offs[1] + 4))          # first hidden bias
    for k in probes:
        h = 1e-3 * max(1.0, abs(float(p[k])))
        pp, pm = p.astype(np.float64).copy(), p.astype(np.float64).copy()
        pp[k] += h
        pm[k] -= h
        lp, _ = mo.loss_and_grad(pp, x, t, L)
        lm, _ = mo.loss_and_grad(pm, x, t, L)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[k]) <= 1e-4 * max(1.0, abs(g[k])), (k, fd, g[k])

"""Learned warm start end to end on a small problem: solutions from the batched
solver, MLP training on the GPU, prediction for a held-out condition.  The
prediction must be closer to the held-out steady state than the free stream,
and a solve started from it must begin with a smaller residual (normalised by
the free-stream run's first iteration) and, run to a 1e-8 drop (FP32 down to
1e-4, FP64 below), reach the lift and drag of the free-stream run within
1e-4: the smooth-limiter scheme has one steady state whatever the start.
(At a 1e-6 drop the two runs still differ by about 2e-4 in CL on this coarse
mesh: the residual is the density change of one iteration, and the slowest
mode decays by only ~1e-4 per iteration, so it understates the distance to
the steady state.)"""
import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d
from gpueularsolver2d_gb300 import warmstart as ws

pytestmark = pytest.mark.gpu


def test_warm_start_small(lib):
    mesh = e2d.Mesh.ogrid(64, 16, seed=1)
    gen = ws.SolverSettings(cfl=3.0, precision=e2d.E2D_FP32)
    train_c = ws.conditions(16, 3, (0.5, 0.65), (-1.0, 3.0))
    held = ws.conditions(1, 4, (0.5, 0.65), (-1.0, 3.0))
    states, _ = ws.generate(mesh, train_c + held, gen, 3000, log=lambda s: None)
    ds = ws.Dataset(mesh, train_c, states[:-1])
    net, loss, _ = ws.train(ds, 600, batch=8192, nhidden=3, lr=2e-3, log=lambda s: None)
    assert loss[-50:].mean() < 0.2 * loss[:10].mean()
    (m, a), w_true = held[0], states[-1]
    p = ws.predict(net, ds, mesh, m, a)
    err_pred = np.abs(p - w_true).mean()
    err_free = np.abs(ws.freestream(m, a, p.shape[0]) - w_true).mean()
    assert err_pred < 0.5 * err_free, (err_pred, err_free)
    ev = ws.SolverSettings(cfl=3.0, precision=e2d.E2D_FP64, switch_resd=1e-4)
    free = ws.run_to_drop(mesh, m, a, ev, 1e-8, 80000)
    warm = ws.run_to_drop(mesh, m, a, ev, 1e-8, 80000, w0=p, epsm=free["epsm"])
    assert free["converged"] and warm["converged"]
    assert warm["first_resd"] < 0.5
    assert abs(warm["cl"] - free["cl"]) < 1e-4
    assert abs(warm["cd"] - free["cd"]) < 1e-4

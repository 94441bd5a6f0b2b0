"""Learned warm start end to end on a small problem: solutions from the batched
solver, MLP training on the GPU (tensor-core kernels), prediction for a
held-out condition.  The prediction must be closer to the held-out steady
state than the free stream, and a solve started from it must begin with a
smaller residual (normalised by the free-stream run's first iteration) and
reach a 1e-8 drop in FP64 with the solver settings of the pipeline (smooth
limiter, K = 10, frozen at Resd 1e-3).  On this coarse 64 x 16 mesh the
limiter is active in many cells, and the values it is frozen at differ
between the two runs, so lift and drag agree within 5e-3 here; on the
pipeline's 256 x 64 mesh they agree within 1e-4 (the pipeline reports the
figure).  The residual is the density change of one iteration and
understates the distance to the steady state (the slowest mode decays by
~1e-4 per iteration), hence the 1e-8 drop.  Training follows the pipeline's
cosine step-size schedule and both runs freeze the limiter values a second
time from the state at 1e-5, as the pipeline does.  The warm run must need at
most 0.7 of the free run's iterations."""
import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d
from gpueularsolver2d_gb300 import warmstart as ws

pytestmark = pytest.mark.gpu


def test_warm_start_small(lib):
    mesh = e2d.Mesh.ogrid(64, 16, seed=1)
    gen = ws.SolverSettings(cfl=3.0, precision=e2d.E2D_FP32)
    train_c = ws.conditions(64, 3, (0.58, 0.68), (-1.0, 3.0))
    held = ws.conditions(1, 4, (0.58, 0.68), (-1.0, 3.0))
    states, _ = ws.generate(mesh, train_c + held, gen, 3000, log=lambda s: None)
    ds = ws.Dataset(mesh, train_c, states[:-1])
    net, loss, _ = ws.train(ds, 4000, batch=8192, nhidden=4, lr=2e-3, lr_final=1e-4, chunk=100,
                            log=lambda s: None)
    assert len(loss) == 4000
    assert loss[-50:].mean() < 0.2 * loss[:10].mean()
    (m, a), w_true = held[0], states[-1]
    p = ws.predict(net, ds, mesh, m, a)
    err_pred = np.abs(p - w_true).mean()
    err_free = np.abs(ws.freestream(m, a, p.shape[0]) - w_true).mean()
    assert err_pred < 0.5 * err_free, (err_pred, err_free)
    ev = ws.SolverSettings(cfl=3.0, precision=e2d.E2D_FP64, refreeze_resd=1e-5)
    free = ws.run_to_drop(mesh, m, a, ev, 1e-8, 80000)
    warm = ws.run_to_drop(mesh, m, a, ev, 1e-8, 80000, w0=p, epsm=free["epsm"])
    assert free["converged"] and warm["converged"]
    for r in (free, warm):  # one history across the two solvers, through 1e-5 to 1e-8
        assert r["iterations_to"]["1e-05"] is not None and r["iterations_to"]["1e-05"] < r["iterations"]
    assert warm["first_resd"] < 0.5
    # the gain: the warm run reaches the drop in at most 0.7 of the free run's
    # iterations (iterations are deterministic, wall time is not)
    print(f"free {free['iterations']} iterations, warm {warm['iterations']}")
    assert warm["iterations"] <= 0.7 * free["iterations"], (warm["iterations"], free["iterations"])
    assert abs(warm["cl"] - free["cl"]) < 5e-3
    assert abs(warm["cd"] - free["cd"]) < 5e-3

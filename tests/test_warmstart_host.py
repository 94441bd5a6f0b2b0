"""Host logic of the warm-start pipeline on the CPU, with the GPU objects
replaced by fakes: the second limiter freeze of ``run_to_drop`` (one history
across two solvers, the second created from the first one's state and
residual norm with its limiter values frozen after its first iteration, and
the first solver's history kept when the second one fails), and the cosine
step-size schedule of ``train``."""
import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d
from gpueularsolver2d_gb300 import warmstart as ws
from gpueularsolver2d_gb300._lib import E2DError

DIVERGED = -5  # E2D_ERR_DIVERGED in include/euler2d.h


class FakeSolver:
    """Stands in for api.Solver: the residual falls by a fixed factor per
    iteration from `start`; `fail_at` raises after that many iterations."""

    created = []
    start, rate, fail_at = 1.0, 0.9, None

    def __init__(self, mesh, params):
        self.params = params
        self.hist = []
        self.state_in = None
        self.norm = None
        self.closed = False
        FakeSolver.created.append(self)

    def set_state(self, w):
        self.state_in = np.array(w)

    def set_residual_norm(self, epsm):
        self.norm = epsm

    def residual_norm(self):
        return 2.5 if self.norm is None else self.norm

    def state(self):
        return np.full((4, 4), float(len(self.hist)))

    def forces(self):
        return 0.25, 0.01

    def history(self):
        return np.array(self.hist)

    def solve(self, max_steps, epsl):
        r = self.hist[-1] if self.hist else self.start / self.rate
        for _ in range(max_steps):
            if FakeSolver.fail_at is not None and len(self.hist) >= FakeSolver.fail_at:
                raise E2DError(DIVERGED, "diverged")
            r *= self.rate
            self.hist.append(r)
            if r <= epsl:
                break
        return np.array(self.hist)

    def close(self):
        self.closed = True


@pytest.fixture
def fake_solver(monkeypatch):
    FakeSolver.created = []
    FakeSolver.start, FakeSolver.rate, FakeSolver.fail_at = 1.0, 0.9, None
    monkeypatch.setattr(ws.e2d, "Solver", FakeSolver)
    return FakeSolver


def expected_iterations(start, rate, level):
    """Iterations of FakeSolver.solve until its residual (start, start * rate,
    ...) is <= level."""
    k, r = 0, start / rate
    while True:
        k += 1
        r *= rate
        if r <= level:
            return k


def test_refreeze_continues_in_a_second_solver(lib, fake_solver):
    settings = ws.SolverSettings(precision=e2d.E2D_FP64, refreeze_resd=1e-5)
    out = ws.run_to_drop(None, 0.6, 1.0, settings, 1e-8, 5000, w0=np.ones((4, 4)), epsm=3.0)
    first, second = fake_solver.created
    n1 = expected_iterations(1.0, 0.9, 1e-5)
    assert len(first.hist) == n1 and first.closed
    # the second solver: the first one's state and residual norm, maxstep
    # reduced by the iterations already run, limiter frozen after one iteration
    assert second.state_in is not None and np.all(second.state_in == n1)
    assert second.norm == 3.0
    assert second.params.maxstep == 5000 - n1
    assert second.params.limiter_freeze_resd == 1.0
    assert first.params.limiter_freeze_resd == settings.freeze_resd
    assert out["converged"]
    assert out["iterations"] == n1 + len(second.hist)
    assert out["iterations_to"]["1e-05"] == n1
    assert out["cl"] == 0.25 and out["start_cl"] == 0.25


def test_no_refreeze_runs_one_solver(lib, fake_solver):
    settings = ws.SolverSettings(precision=e2d.E2D_FP64)
    out = ws.run_to_drop(None, 0.6, 1.0, settings, 1e-8, 5000)
    assert len(fake_solver.created) == 1
    assert out["iterations"] == expected_iterations(1.0, 0.9, 1e-8)
    assert out["converged"] and np.isnan(out["start_cl"])


def test_refreeze_failure_keeps_the_whole_history(lib, fake_solver, monkeypatch):
    class FailSecond(FakeSolver):
        def solve(self, max_steps, epsl):
            if len(FakeSolver.created) == 2:  # the second solver runs 20 iterations, then fails
                self.hist = [1e-5] * 20
                raise E2DError(DIVERGED, "diverged")
            return super().solve(max_steps, epsl)

    monkeypatch.setattr(ws.e2d, "Solver", FailSecond)
    settings = ws.SolverSettings(precision=e2d.E2D_FP64, refreeze_resd=1e-5)
    out = ws.run_to_drop(None, 0.6, 1.0, settings, 1e-8, 5000)
    n1 = expected_iterations(1.0, 0.9, 1e-5)
    assert len(FakeSolver.created) == 2
    assert not out["converged"] and np.isnan(out["cl"])
    assert out["iterations"] == n1 + 20


class FakeMLP:
    """Stands in for api.MLP: records the step sizes and chunk lengths."""

    last = None

    def __init__(self, nhidden, batch, seed, lr):
        self.lr0 = lr
        self.lrs, self.chunks = [], []
        FakeMLP.last = self

    def set_data(self, x, t):
        pass

    def set_lr(self, lr):
        self.lrs.append(lr)

    def train(self, steps, record_loss=True):
        self.chunks.append(steps)
        return np.full(steps, 0.5)


class FakeDataset:
    x = np.zeros((8, 32), np.float32)
    t = np.zeros((8, 4), np.float32)


def test_cosine_step_size_schedule(lib, monkeypatch):
    monkeypatch.setattr(ws.e2d, "MLP", FakeMLP)
    net, loss, _ = ws.train(FakeDataset(), 1030, batch=2048, lr=1e-3, lr_final=1e-5, chunk=100,
                            log=lambda s: None)
    assert len(loss) == 1030
    assert net.chunks == [100] * 10 + [30]
    lrs = np.array(net.lrs)
    assert len(lrs) == 11 and np.all(np.diff(lrs) < 0)
    # the step size of each chunk is the cosine at the chunk's midpoint
    mid = (np.arange(11) * 100 + 0.5 * np.array([100] * 10 + [30])) / 1030
    np.testing.assert_allclose(lrs, 1e-5 + 0.5 * (1e-3 - 1e-5) * (1 + np.cos(np.pi * mid)), rtol=1e-12)
    assert 1e-5 < lrs[-1] < 1.01e-5 + 1e-6 and 0.99e-3 < lrs[0] < 1e-3


def test_constant_step_size_without_lr_final(lib, monkeypatch):
    monkeypatch.setattr(ws.e2d, "MLP", FakeMLP)
    net, loss, _ = ws.train(FakeDataset(), 700, batch=2048, lr=2e-3, log=lambda s: None)
    assert net.lrs == [] and net.chunks == [700] and net.lr0 == 2e-3 and len(loss) == 700


def test_physical():
    w = ws.freestream(0.6, 1.0, 10)
    assert ws.physical(w)
    for i, v in [(0, 0.0), (0, float("nan")), (3, 0.1), (1, float("inf"))]:
        bad = w.copy()
        bad[4, i] = v
        assert not ws.physical(bad), (i, v)


def test_warm_run_without_fallback(lib, fake_solver):
    settings = ws.SolverSettings(precision=e2d.E2D_FP64)
    out = ws.run_warm(None, 0.6, 1.0, settings, 1e-8, 5000, ws.freestream(0.6, 1.0, 4), epsm=2.0)
    assert out["fallback"] is None and out["converged"]
    assert len(fake_solver.created) == 1 and fake_solver.created[0].state_in is not None


def test_unphysical_prediction_falls_back_to_the_free_stream(lib, fake_solver):
    settings = ws.SolverSettings(precision=e2d.E2D_FP64)
    w = ws.freestream(0.6, 1.0, 4)
    w[2, 0] = -1.0
    out = ws.run_warm(None, 0.6, 1.0, settings, 1e-8, 5000, w, epsm=2.0)
    assert out["fallback"] == "prediction not physical" and out["converged"]
    (only,) = fake_solver.created
    assert only.state_in is None and only.norm == 2.0  # started from the free stream, same normalisation


def test_diverged_warm_run_falls_back_and_counts_its_cost(lib, fake_solver, monkeypatch):
    class DivergeFirst(FakeSolver):
        def solve(self, max_steps, epsl):
            if len(FakeSolver.created) == 1:  # the warm run: 40 iterations, then diverges
                self.hist = [0.5] * 40
                raise E2DError(DIVERGED, "diverged")
            return super().solve(max_steps, epsl)

    monkeypatch.setattr(ws.e2d, "Solver", DivergeFirst)
    settings = ws.SolverSettings(precision=e2d.E2D_FP64)
    out = ws.run_warm(None, 0.6, 1.0, settings, 1e-8, 5000, ws.freestream(0.6, 1.0, 4), epsm=2.0)
    warm, free = FakeSolver.created
    assert warm.state_in is not None and free.state_in is None
    assert out["fallback"].startswith("warm run failed") and out["converged"]
    assert out["iterations"] == 40 + len(free.hist)
    assert out["failed_attempt"]["iterations"] == 40
    # levels reached count the failed attempt's iterations too
    assert all(v is None or v > 40 for v in out["iterations_to"].values())
    assert out["iterations_to"]["1e-05"] > 40
    assert out["start_cl"] == 0.25  # the prediction's, from the warm attempt

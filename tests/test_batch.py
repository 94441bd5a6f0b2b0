"""Batched cases (e2d_batch_*): every case of a batch must give the same result,
bit for bit, as a single-case solver with the same parameters and block size
-- state and residual history -- whatever the launch shape, and each case must
stop on its own residual test."""
import os
import tempfile

import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d

pytestmark = pytest.mark.gpu

SIZES = [(32, 8, 1), (48, 12, 2), (64, 16, 3), (40, 10, 4), (24, 6, 5)]
FLOWS = [(0.5, 1.25, 1.5), (0.6, -1.0, 1.2), (0.4, 3.0, 2.0), (0.7, 0.5, 1.5), (0.55, 2.0, 1.0)]


def make_cases(prec):
    meshes = [e2d.Mesh.ogrid(ni, nj, seed=s) for ni, nj, s in SIZES]
    params = [e2d.default_params(ma=m, alpha_deg=a, cfl=c, precision=prec, ordering=e2d.E2D_ORDER_MORTON,
                                 maxstep=400) for m, a, c in FLOWS]
    return meshes, params


@pytest.mark.parametrize("prec", [e2d.E2D_FP64, e2d.E2D_FP32])
def test_batch_equals_single_cases(lib, prec):
    meshes, params = make_cases(prec)
    b = e2d.Batch(meshes, params)
    ncase, ntot, npad = b.info()
    assert ncase == len(SIZES) and ntot == sum(2 * ni * nj for ni, nj, _ in SIZES) and npad % 256 == 0
    b.step(17)
    for c, (m, p) in enumerate(zip(meshes, params)):
        s = e2d.Solver(m, p)
        s.step(17)
        assert np.array_equal(b.state(c), s.state()), c
        assert np.array_equal(b.history(c), s.history()), c


def test_batch_options_equal_single_cases(lib):
    """Per-case options in one batch: global time step (a per-case minimum),
    the far-field fix at M 1.5, the Venkatakrishnan limiter and a residual-level
    limiter freeze, each equal to its own single-case run."""
    meshes = [e2d.Mesh.ogrid(ni, nj, seed=s) for ni, nj, s in SIZES[:4]]
    params = [e2d.default_params(ma=0.5, alpha_deg=1.0, cfl=1.5, global_dt=1),
              e2d.default_params(ma=1.5, alpha_deg=0.0, cfl=1.0, far_field_fix=1),
              e2d.default_params(ma=0.6, alpha_deg=2.0, cfl=2.0, limiter=1, limiter_k=3.0),
              e2d.default_params(ma=0.6, alpha_deg=1.0, cfl=1.5, limiter_freeze_resd=0.5, global_dt=1)]
    for p in params:
        p.ordering = e2d.E2D_ORDER_MORTON
    b = e2d.Batch(meshes, params)
    b.step(21)
    for c, (m, p) in enumerate(zip(meshes, params)):
        s = e2d.Solver(m, p)
        s.step(21)
        assert np.array_equal(b.state(c), s.state()), c
        assert np.array_equal(b.history(c), s.history()), c


def test_batch_tuned_order_and_shape(lib, tmp_path):
    """The autotuner picks a cell order and launch shape; the tuned batch gives
    the same bits as a plain batch (the order only changes the layout), and
    the cache holds one entry per order."""
    meshes, params = make_cases(e2d.E2D_FP32)
    cache = str(tmp_path / "tune.json")
    t = e2d.Batch.tuned(meshes, params, cache, iters=8)
    assert t.ordering in (e2d.E2D_ORDER_MORTON, e2d.E2D_ORDER_RCM, e2d.E2D_ORDER_FILE)
    assert open(cache).read().count("|order=") == 3
    ref = e2d.Batch(meshes, params)
    t.step(9)
    ref.step(9)
    for c in range(len(meshes)):
        assert np.array_equal(t.state(c), ref.state(c)), c
    t2 = e2d.Batch.tuned(meshes, params, cache, iters=8)  # from the cache
    assert t2.ordering == t.ordering and t2.launch() == t.launch()


def test_batch_launch_shapes_agree(lib):
    meshes, params = make_cases(e2d.E2D_FP64)
    ref = e2d.Batch(meshes, params)
    ref.step(9)
    for block, grid in [(64, 0), (256, 0), (128, 7), (64, 3)]:
        b = e2d.Batch(meshes, params)
        b.set_launch(block, grid)
        assert b.launch()[0] == block
        b.step(9)
        for c in range(len(meshes)):
            # the state does not depend on the launch shape; the residual
            # partials group by block size, so histories agree to rounding
            assert np.array_equal(b.state(c), ref.state(c)), (block, grid, c)
            np.testing.assert_allclose(b.history(c), ref.history(c), rtol=1e-12)


def test_batch_cases_stop_on_their_own(lib):
    meshes, params = make_cases(e2d.E2D_FP64)
    singles = []
    for m, p in zip(meshes, params):
        s = e2d.Solver(m, p)
        s.step(120)
        singles.append(s.history())
    epsl = float(np.median([h[60] for h in singles]))
    want = [int(np.argmax(h <= epsl)) + 1 if (h <= epsl).any() else 120 for h in singles]
    assert len(set(want)) > 1
    b = e2d.Batch(meshes, params)
    n = b.solve(120, epsl)
    assert list(n) == want
    for c, (m, p) in enumerate(zip(meshes, params)):
        s = e2d.Solver(m, p)
        s.solve(120, epsl)
        assert np.array_equal(b.state(c), s.state()), c
        assert b.progress(c)[2] == 1


def test_batch_autotune_restores_state_and_caches(lib):
    meshes, params = make_cases(e2d.E2D_FP32)
    b = e2d.Batch(meshes, params)
    b.step(5)
    before = [b.state(c) for c in range(len(meshes))]
    hist = [b.history(c) for c in range(len(meshes))]
    with tempfile.TemporaryDirectory() as d:
        cache = os.path.join(d, "tune.json")
        block, grid, ms = b.autotune(cache, iters=8)
        assert block in (64, 128, 256) and grid >= 1 and ms > 0
        assert b.launch() == (block, grid)
        for c in range(len(meshes)):
            assert np.array_equal(b.state(c), before[c])
            assert np.array_equal(b.history(c), hist[c])
        text = open(cache).read()
        assert text.strip().startswith("{") and "cases=5" in text
        b2 = e2d.Batch(meshes, params)
        assert b2.autotune(cache, iters=8) == (block, grid, pytest.approx(ms))
    # the tuned batch still matches the single-case solvers
    b.step(6)
    for c, (m, p) in enumerate(zip(meshes, params)):
        s = e2d.Solver(m, p)
        s.step(11)
        assert np.array_equal(b.state(c), s.state()), c

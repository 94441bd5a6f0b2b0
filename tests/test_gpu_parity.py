"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

The FP64 variant must reproduce the oracle bit for bit (same IEEE operations,
no FMA contraction); the FP32 variant is reported against the FP64 run of the
same code with the tolerance written in each test.
"""
import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d

pytestmark = pytest.mark.gpu

BLAZEK5 = [0.0695, 0.1602, 0.2898, 0.5060, 1.0]


def run_pair(mesh, oracle, nsteps, **kw):
    p = e2d.default_params(**kw)
    s = e2d.Solver(mesh, p)
    x, y, tri = mesh.nodes()
    c = oracle.Case(x, y, tri, oracle.params_from_e2d(p))
    r_ref = c.run(nsteps)
    s.step(nsteps)
    return s, c, r_ref


@pytest.mark.parametrize("kw", [
    dict(ma=0.5, alpha_deg=1.25, cfl=1.5),
    dict(ma=0.8, alpha_deg=1.25, cfl=2.0, irs_eps=0.6, rk_stages=5, rk_coef=BLAZEK5),
    dict(ma=0.5, alpha_deg=-2.0, cfl=1.0, irs_sweeps=0),
    dict(ma=0.7, alpha_deg=3.0, cfl=1.5, irs_sweeps=3, ordering=e2d.E2D_ORDER_MORTON),
    dict(ma=0.6, alpha_deg=1.0, cfl=1.5, limiter_freeze=12, ordering=e2d.E2D_ORDER_MORTON),
    dict(ma=0.7, alpha_deg=2.0, cfl=2.0, limiter=1, limiter_k=3.0, ordering=e2d.E2D_ORDER_MORTON),
    dict(ma=0.6, alpha_deg=1.0, cfl=1.5, limiter_freeze_resd=0.5, ordering=e2d.E2D_ORDER_MORTON),
    dict(ma=0.5, alpha_deg=1.0, cfl=1.5, global_dt=1, ordering=e2d.E2D_ORDER_MORTON),
    dict(ma=1.5, alpha_deg=0.0, cfl=1.0, far_field_fix=1, ordering=e2d.E2D_ORDER_MORTON),
    dict(ma=0.6, alpha_deg=1.0, cfl=1.5, ordering=e2d.E2D_ORDER_RCM),
    dict(ma=0.7, alpha_deg=2.0, cfl=1.5, first_order_iters=10, ordering=e2d.E2D_ORDER_MORTON),
    dict(ma=0.8, alpha_deg=1.25, cfl=2.0, limiter=2, ordering=e2d.E2D_ORDER_MORTON),
    dict(ma=0.7, alpha_deg=2.0, cfl=1.5, limiter=3, limiter_k=5.0, limiter_freeze=15, ordering=e2d.E2D_ORDER_RCM),
    dict(ma=0.8, alpha_deg=1.25, cfl=2.0, positivity_fix=1, first_order_iters=3, ordering=e2d.E2D_ORDER_MORTON),
])
def test_fp64_bit_exact_vs_oracle(lib, oracle, kw):
    mesh = e2d.Mesh.ogrid(48, 12, seed=7)
    s, c, r_ref = run_pair(mesh, oracle, 25, **kw)
    w = s.state()
    assert np.array_equal(w, c.state()), np.max(np.abs(w - c.state()))
    hist = s.history()
    assert len(hist) == 25
    np.testing.assert_allclose(hist, r_ref, rtol=1e-12, atol=0)


@pytest.mark.parametrize("ordering", [e2d.E2D_ORDER_FILE, e2d.E2D_ORDER_MORTON])
def test_fp64_bit_exact_partial_tile(lib, oracle, ordering):
    """A mesh whose cell count is not a multiple of the 128-cell tile (50 x 13
    O-grid: 1300 cells, the last tile 20 cells): the FP64 passes that work in
    tiles (pass A's once-per-face spectral radii and warp-shared limiter
    divisions, pass B's once-per-face Roe fluxes) run padding lanes there."""
    mesh = e2d.Mesh.ogrid(50, 13, seed=4)
    s, c, r_ref = run_pair(mesh, oracle, 30, ma=0.75, alpha_deg=2.0, cfl=1.5, ordering=ordering)
    assert mesh.info().ncell % 128 != 0
    assert np.array_equal(s.state(), c.state()), np.max(np.abs(s.state() - c.state()))
    np.testing.assert_allclose(s.history(), r_ref, rtol=1e-12, atol=0)


def test_fp64_bit_exact_128x32_morton(lib, oracle):
    mesh = e2d.Mesh.ogrid(128, 32, seed=1)
    s, c, r_ref = run_pair(mesh, oracle, 40, ma=0.5, alpha_deg=1.25, cfl=2.0,
                           ordering=e2d.E2D_ORDER_MORTON)
    assert np.array_equal(s.state(), c.state())
    np.testing.assert_allclose(s.history(), r_ref, rtol=1e-12)


def test_fp32_error_vs_fp64(lib):
    """FP32 stencil against the FP64 run of the same code, early in the run.

    One iteration stays at FP32 rounding, ten within 1e-4.  Later in the
    start-up transient the limiter and the smoothing clamp switch on tiny
    differences and amplify any change of rounding (the reference's own
    FMA-contracted FP64 kernels drift from the oracle the same way, at the
    FP64 level), so the comparison that matters is the converged one below."""
    mesh = e2d.Mesh.ogrid(128, 32, seed=1)
    kw = dict(ma=0.5, alpha_deg=1.25, cfl=2.0)
    s64 = e2d.Solver(mesh, e2d.default_params(**kw))
    s32 = e2d.Solver(mesh, e2d.default_params(precision=e2d.E2D_FP32, **kw))

    def err():
        w64, w32 = s64.state(), s32.state()
        return (np.abs(w32 - w64) / np.abs(w64).max(axis=0)).max()

    s64.step(1)
    s32.step(1)
    assert err() < 5e-6
    s64.step(9)
    s32.step(9)
    assert err() < 1e-4


def test_fp32_converged_solution_vs_fp64(lib):
    """Converged FP32 and FP64 solutions of the same case (smooth limiter,
    K = 20, so that both converge to one steady state): the FP32 state stalls
    near its rounding floor (~1e-5 drop), FP64 goes on to 1e-6.  Tolerances:
    state 1e-4 max / 1e-5 median relative to each component's largest
    magnitude, CL and CD within 1e-5."""
    mesh = e2d.Mesh.ogrid(128, 32, seed=1)
    kw = dict(ma=0.5, alpha_deg=1.25, cfl=3.0, limiter=1, limiter_k=20.0, ordering=e2d.E2D_ORDER_MORTON,
              maxstep=40000)
    s64 = e2d.Solver(mesh, e2d.default_params(**kw))
    h64 = s64.solve(40000, 1e-6)
    assert h64[-1] <= 1e-6
    s32 = e2d.Solver(mesh, e2d.default_params(precision=e2d.E2D_FP32, **kw))
    h32 = s32.solve(20000, 1e-6)
    assert h32[-1] < 1e-4
    w64, w32 = s64.state(), s32.state()
    d = np.abs(w32 - w64) / np.abs(w64).max(axis=0)
    assert d.max() < 1e-4 and np.median(d) < 1e-5, (d.max(), np.median(d))
    (cl64, cd64), (cl32, cd32) = s64.forces(), s32.forces()
    assert abs(cl32 - cl64) < 1e-5 and abs(cd32 - cd64) < 1e-5, (cl32 - cl64, cd32 - cd64)


def test_set_precision_continues_the_run(lib):
    """Switching FP32 -> FP64 part way equals saving the FP32 state and
    residual norm and continuing in a fresh FP64 solver, bit for bit; the
    history runs on across the switch."""
    mesh = e2d.Mesh.ogrid(48, 12, seed=7)
    kw = dict(ma=0.6, alpha_deg=1.0, cfl=1.5, ordering=e2d.E2D_ORDER_MORTON)
    a = e2d.Solver(mesh, e2d.default_params(precision=e2d.E2D_FP32, **kw))
    a.step(40)
    w, epsm, h32 = a.state(), a.residual_norm(), a.history()
    a.set_precision(e2d.E2D_FP64)
    assert np.array_equal(a.state(), w)
    a.step(25)
    c = e2d.Solver(mesh, e2d.default_params(**kw))
    c.set_state(w)
    c.set_residual_norm(epsm)
    c.step(25)
    assert np.array_equal(a.state(), c.state())
    h = a.history()
    assert len(h) == 65 and np.array_equal(h[:40], h32) and np.array_equal(h[40:], c.history())
    a.set_precision(e2d.E2D_FP32)  # and back down: the state rounds to FP32
    assert np.allclose(a.state(), c.state(), rtol=1e-6, atol=0)
    a.step(1)
    with pytest.raises(Exception):
        a.set_precision(7)
    frozen = e2d.Solver(mesh, e2d.default_params(limiter_freeze=1, precision=e2d.E2D_FP32, **kw))
    frozen.step(2)
    with pytest.raises(Exception, match="frozen"):
        frozen.set_precision(e2d.E2D_FP64)


def test_solve_stops_like_reference_loop(lib, oracle):
    mesh = e2d.Mesh.ogrid(32, 8, seed=3)
    p = e2d.default_params(ma=0.5, alpha_deg=1.25, cfl=1.5)
    s = e2d.Solver(mesh, p)
    x, y, tri = mesh.nodes()
    c = oracle.Case(x, y, tri, oracle.params_from_e2d(p))
    full = c.run(200)
    epsl = float(full[120])  # stop exactly where the reference loop would
    s2 = e2d.Solver(mesh, p)
    hist = s2.solve(500, epsl)
    k = int(np.argmax(full <= epsl)) + 1
    assert len(hist) == k
    np.testing.assert_allclose(hist, full[:k], rtol=1e-12)
    # a second solve with the same target runs nothing (Resd already <= EPSL)
    assert len(s2.solve(10, epsl)) == 0


def test_split_steps_equal_one_run(lib):
    mesh = e2d.Mesh.ogrid(40, 10, seed=5)
    p = e2d.default_params(ma=0.6, alpha_deg=2.0, cfl=1.5, graph_iters=4)
    a = e2d.Solver(mesh, p)
    b = e2d.Solver(mesh, p)
    a.step(11)
    for n in (3, 1, 7):
        b.step(n)
    assert np.array_equal(a.state(), b.state())
    assert np.array_equal(a.history(), b.history())


def test_ordering_invariance(lib):
    # the per-cell arithmetic does not depend on the cell order
    mesh = e2d.Mesh.ogrid(96, 24, seed=11)
    for prec in (e2d.E2D_FP64, e2d.E2D_FP32):
        kw = dict(ma=0.75, alpha_deg=1.0, cfl=2.0, precision=prec)
        a = e2d.Solver(mesh, e2d.default_params(ordering=e2d.E2D_ORDER_FILE, **kw))
        b = e2d.Solver(mesh, e2d.default_params(ordering=e2d.E2D_ORDER_MORTON, **kw))
        a.step(20)
        b.step(20)
        assert np.array_equal(a.state(), b.state())


def test_state_roundtrip_and_forces(lib):
    mesh = e2d.Mesh.ogrid(64, 16, seed=2)
    s = e2d.Solver(mesh, e2d.default_params(ma=0.5, alpha_deg=2.0, cfl=1.5))
    s.step(30)
    w = s.state()
    s2 = e2d.Solver(mesh, e2d.default_params(ma=0.5, alpha_deg=2.0, cfl=1.5))
    s2.set_state(w)
    assert np.array_equal(s2.state(), w)
    cl, cd = s.forces()
    assert np.isfinite(cl) and np.isfinite(cd)


@pytest.mark.parametrize("prec", [e2d.E2D_FP64, e2d.E2D_FP32])
def test_positivity_fix_on_cold_cells(lib, oracle, prec):
    """The positivity fallback on a start state with cold cells (faces with
    negative reconstructed pressure): FP64 equals the oracle bit for bit over
    10 iterations, FP32 runs to the same finite state within 1e-3; without the
    option the solver reports the divergence."""
    from test_oracle_options import cold_cells_state
    mesh = e2d.Mesh.ogrid(48, 12, seed=7)
    w0 = cold_cells_state(oracle, mesh)
    p = e2d.default_params(ma=0.8, alpha_deg=1.25, cfl=1.0, positivity_fix=1, precision=prec)
    s = e2d.Solver(mesh, p)
    s.set_state(w0)
    s.step(10)
    x, y, tri = mesh.nodes()
    c = oracle.Case(x, y, tri, oracle.params_from_e2d(e2d.default_params(ma=0.8, alpha_deg=1.25, cfl=1.0,
                                                                        positivity_fix=1)))
    c.set_state(w0)
    c.run(10)
    if prec == e2d.E2D_FP64:
        assert np.array_equal(s.state(), c.state())
    else:
        assert np.max(np.abs(s.state() - c.state())) / np.max(np.abs(c.state())) < 1e-3
    q = e2d.Solver(mesh, e2d.default_params(ma=0.8, alpha_deg=1.25, cfl=1.0, precision=prec))
    q.set_state(w0)
    with pytest.raises(Exception, match="diverged|non-positive|NaN"):
        q.step(10)


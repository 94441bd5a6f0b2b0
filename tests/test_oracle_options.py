"""Scheme options of the oracle that have no reference counterpart (CPU).

global_dt: every cell advances with the smallest local step of the mesh (the
intent of the reference's disabled kernel_TimeStep, gpu_solver.cu:880-936).
far_field_fix: the supersonic test of the far-field boundary
(gpu_solver.cu:79) compares the non-dimensional normal velocity with the
non-dimensional free-stream sound speed 1/M instead of the dimensional AIN.
The GPU kernels are checked against these oracle paths bit for bit in
test_gpu_parity.py."""
import numpy as np

import gpueularsolver2d_gb300 as e2d


def _case(oracle, mesh, **kw):
    x, y, tri = mesh.nodes()
    return oracle.Case(x, y, tri, oracle.params(**kw))


def test_global_dt_is_min_of_local(lib, oracle):
    mesh = e2d.Mesh.ogrid(32, 8, seed=3)
    loc = _case(oracle, mesh, ma=0.6, alpha_deg=1.0, cfl=1.5)
    glo = _case(oracle, mesh, ma=0.6, alpha_deg=1.0, cfl=1.5, global_dt=1)
    loc.run(3)
    glo.set_state(loc.state())
    a, b = loc.stage_probe(), glo.stage_probe()
    assert np.all(b["dt"] == a["dt"].min())
    assert a["dt"].max() > 10 * a["dt"].min()  # the option does change the step
    np.testing.assert_array_equal(a["res"], b["res"])


def test_global_dt_runs_and_converges_slower(lib, oracle):
    mesh = e2d.Mesh.ogrid(32, 8, seed=3)
    loc = _case(oracle, mesh, ma=0.5, alpha_deg=1.0, cfl=1.5)
    glo = _case(oracle, mesh, ma=0.5, alpha_deg=1.0, cfl=1.5, global_dt=1)
    rl, rg = loc.run(60), glo.run(60)
    assert np.all(np.isfinite(rg)) and rl[-1] < rg[-1]


def test_far_field_fix_supersonic_branch(lib, oracle):
    mesh = e2d.Mesh.ogrid(32, 8, seed=3)
    ma = 1.5
    fix = _case(oracle, mesh, ma=ma, alpha_deg=0.0, far_field_fix=1)
    ref = _case(oracle, mesh, ma=ma, alpha_deg=0.0)
    g, T, R = 1.4, 288.15, 287.06
    ain = np.sqrt(g * R * T)
    rho_e = R * T / (ma * ain) ** 2 / (g - 1) + 0.5
    dw = np.array([1.02, 0.98, 0.01, rho_e * 1.01])
    # outflow face, normal +x (nx = vectory / |v|): ghost = interior state
    np.testing.assert_array_equal(fix.far_ghost(dw, 0.0, 0.3), dw)
    # inflow face, normal -x: ghost = free stream
    np.testing.assert_array_equal(fix.far_ghost(dw, 0.0, -0.3), [1.0, 1.0, 0.0, rho_e])
    # the reference test never takes the supersonic branch
    assert not np.array_equal(ref.far_ghost(dw, 0.0, 0.3), dw)
    # a face whose normal velocity is subsonic keeps the characteristic branch
    np.testing.assert_array_equal(fix.far_ghost(dw, 0.3, 0.0), ref.far_ghost(dw, 0.3, 0.0))


def test_far_field_fix_inactive_when_subsonic(lib, oracle):
    mesh = e2d.Mesh.ogrid(32, 8, seed=3)
    a = _case(oracle, mesh, ma=0.6, alpha_deg=2.0, cfl=1.5)
    b = _case(oracle, mesh, ma=0.6, alpha_deg=2.0, cfl=1.5, far_field_fix=1)
    np.testing.assert_array_equal(a.run(10), b.run(10))
    np.testing.assert_array_equal(a.state(), b.state())


def cold_cells_state(oracle, mesh, seed=1, lo=0.05):
    """Free stream with every 12th interior cell (away from the boundary)
    made dense-deficient and nearly pressureless: limited reconstructions
    toward those cells give faces with negative pressure."""
    c = _case(oracle, mesh, ma=0.8, alpha_deg=1.25, cfl=1.0)
    ei, ed, ci, cd = c.topology()
    inner = (ci[:, 0] == 3) & np.all(ci[np.maximum(ci[:, 4:7], 1) - 1, 0] == 3, axis=1)
    rng = np.random.default_rng(seed)
    cand = np.flatnonzero(inner)
    idx = rng.choice(cand, len(cand) // 12, replace=False)
    w = c.state()
    w[idx, 0] *= rng.uniform(0.5, 1.0, len(idx))
    w[idx, 3] = 0.5 * (w[idx, 1] ** 2 + w[idx, 2] ** 2) / w[idx, 0] + rng.uniform(lo, 2 * lo, len(idx))
    return w


def test_positivity_fix_keeps_faces_physical(lib, oracle):
    """Option positivity_fix: a face side whose limited reconstruction has a
    non-positive density or pressure takes the cell state.  From a state with
    cold cells the reference reconstruction gives NaN fluxes after one
    iteration; with the option every flux is finite and the run continues."""
    mesh = e2d.Mesh.ogrid(48, 12, seed=7)
    w = cold_cells_state(oracle, mesh)
    ref = _case(oracle, mesh, ma=0.8, alpha_deg=1.25, cfl=1.0)
    fix = _case(oracle, mesh, ma=0.8, alpha_deg=1.25, cfl=1.0, positivity_fix=1)
    ref.set_state(w)
    fix.set_state(w)
    pr, pf = ref.stage_probe(), fix.stage_probe()
    assert np.isnan(pr["flux"]).any() and np.isfinite(pf["flux"]).all()
    r = fix.run(10)
    assert len(r) == 10 and np.all(np.isfinite(r)) and np.all(np.isfinite(fix.state()))
    # on the free stream (nothing to fix) the option changes nothing
    a = _case(oracle, mesh, ma=0.6, alpha_deg=1.0, cfl=1.5)
    b = _case(oracle, mesh, ma=0.6, alpha_deg=1.0, cfl=1.5, positivity_fix=1)
    np.testing.assert_array_equal(a.run(5), b.run(5))
    np.testing.assert_array_equal(a.state(), b.state())


def test_first_order_iters(lib, oracle):
    """Option first_order_iters = k: the first k iterations use the cell states
    on every face (first order, like the reference's boundary faces), then the
    limited reconstruction."""
    mesh = e2d.Mesh.ogrid(32, 8, seed=3)
    kw = dict(ma=0.6, alpha_deg=1.0, cfl=1.5)
    ref, f2, f5 = (_case(oracle, mesh, **kw, first_order_iters=k) for k in (0, 2, 5))
    r2, r5, rr = f2.run(2), f5.run(2), ref.run(2)
    np.testing.assert_array_equal(f2.state(), f5.state())  # both first order so far
    assert not np.array_equal(f2.state(), ref.state())
    f2.run(1)
    f5.run(1)
    assert not np.array_equal(f2.state(), f5.state())  # iteration 3: f2 second order, f5 first
    # a first-order iteration's face states are the cell states: the probe's
    # fluxes do not depend on the gradients
    p = f5.stage_probe()
    assert np.all(np.isfinite(p["flux"]))


def test_cell_limiters_bound_the_face_states(lib, oracle):
    """Cell-wise limiter options (2: min over the cell's interior faces of the
    reference's per-face value, 3: the same with the Venkatakrishnan form):
    with option 2 every reconstructed face state lies inside the cell's
    neighbour bounds, like the per-face reference limiter; both change the
    solution."""
    mesh = e2d.Mesh.ogrid(32, 8, seed=3)
    kw = dict(ma=0.7, alpha_deg=2.0, cfl=1.5)
    ref = _case(oracle, mesh, **kw)
    ref.run(20)
    w = ref.state()
    for lim in (2, 3):
        c = _case(oracle, mesh, **kw, limiter=lim, limiter_k=5.0)
        c.set_state(w)
        p = c.stage_probe()
        assert np.all(np.isfinite(p["flux"]))
        q = _case(oracle, mesh, **kw, limiter=lim, limiter_k=5.0)
        q.run(20)
        assert not np.array_equal(q.state(), w)

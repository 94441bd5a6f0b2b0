"""Host-side logic of libeuler2d (no GPU needed): the C ABI loads and exports
every symbol the header declares, the mesh reader/writer and generator, the
O(N) set-up against the oracle's restatement of CalculationMeshGeo +
changeEdge, the Morton permutation, and error reporting."""
import os
import re
import tempfile

import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d
from gpueularsolver2d_gb300 import _lib
from conftest import ROOT, reference_mesh


def header_functions(name):
    text = open(os.path.join(ROOT, "include", name)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(e2d_\w+)\s*\(", text)))


def test_library_exports_every_declared_symbol(lib):
    fns = header_functions("euler2d.h")
    assert len(fns) > 20
    for f in fns:
        assert hasattr(lib, f), f
        assert f in _lib.SIGNATURES, f


@pytest.mark.parametrize("ni,nj,seed", [(16, 4, 1), (48, 12, 7), (128, 32, 1), (100, 20, 42)])
def test_setup_matches_oracle(lib, oracle, ni, nj, seed):
    mesh = e2d.Mesh.ogrid(ni, nj, seed=seed)
    x, y, tri = mesh.nodes()
    case = oracle.Case(x, y, tri, oracle.params())
    for a, b in zip(mesh.topology(), case.topology()):
        assert np.array_equal(a, b)
    assert np.array_equal(mesh.order(e2d.E2D_ORDER_MORTON) + 1, case.morton())
    assert np.array_equal(mesh.order(e2d.E2D_ORDER_RCM) + 1, case.rcm())
    assert np.array_equal(mesh.order(e2d.E2D_ORDER_FILE), np.arange(case.ncell))


@pytest.mark.parametrize("name", ["2822-3k.dat", "2822-1w.dat", "2822-5w.dat", "2822-9w.dat"])
def test_setup_matches_oracle_on_reference_meshes(lib, oracle, name):
    path = reference_mesh(name)
    if path is None:
        pytest.skip("reference meshes not available")
    mesh = e2d.Mesh.read(path)
    case = oracle.Case.from_file(path, oracle.params())
    for a, b in zip(mesh.topology(), case.topology()):
        assert np.array_equal(a, b)
    assert np.array_equal(mesh.order(e2d.E2D_ORDER_MORTON) + 1, case.morton())
    assert np.array_equal(mesh.order(e2d.E2D_ORDER_RCM) + 1, case.rcm())


def test_rcm_is_a_banded_permutation(lib):
    """RCM is a permutation whose neighbour index distance (bandwidth) is far
    below the cell count on an O-grid."""
    mesh = e2d.Mesh.ogrid(96, 24, seed=4)
    perm = mesh.order(e2d.E2D_ORDER_RCM)
    n = len(perm)
    assert np.array_equal(np.sort(perm), np.arange(n))
    pos = np.empty(n, np.int64)
    pos[perm] = np.arange(n)
    _, _, ci, _ = mesh.topology()
    nb = ci[:, 4:7].reshape(-1) - 1
    i = np.repeat(np.arange(n), 3)
    ok = nb >= 0
    band = np.abs(pos[i[ok]] - pos[nb[ok]]).max()
    assert band < n // 8, band


def test_ogrid_sizes_and_tags(lib):
    for ni, nj in [(16, 4), (128, 32), (256, 64)]:
        inf = e2d.Mesh.ogrid(ni, nj).info()
        assert (inf.ncell, inf.nnode, inf.nedge, inf.nwall, inf.nfar) == (
            2 * ni * nj, ni * (nj + 1), 3 * ni * nj + ni, ni, ni)


def test_ogrid_deterministic_and_ccw(lib):
    a = e2d.Mesh.ogrid(64, 16, seed=5).nodes()
    b = e2d.Mesh.ogrid(64, 16, seed=5).nodes()
    c = e2d.Mesh.ogrid(64, 16, seed=6).nodes()
    assert all(np.array_equal(u, v) for u, v in zip(a, b))
    assert not np.array_equal(a[0], c[0])
    x, y, tri = a
    t = tri - 1
    area = 0.5 * ((y[t[:, 2]] - y[t[:, 0]]) * (x[t[:, 1]] - x[t[:, 0]])
                  - (y[t[:, 1]] - y[t[:, 0]]) * (x[t[:, 2]] - x[t[:, 0]]))
    assert area.min() > 0
    r = np.hypot(x - 0.5, y)
    assert abs(r.max() - 20.0) < 1e-9


def test_mesh_write_read_roundtrip(lib):
    m = e2d.Mesh.ogrid(32, 8, seed=2)
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "m.dat")
        m.write(p)
        m2 = e2d.Mesh.read(p)
    for u, v in zip(m.nodes(), m2.nodes()):
        assert np.array_equal(u, v)


def test_input_read(lib):
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "input.dat")
        with open(p, "w") as f:
            f.write("0.8 1.25 1.4 101325 288.15 4.0 1e-6 5000\n")
        prm = e2d.read_input(p)
        assert (prm.ma, prm.alpha_deg, prm.cfl, prm.epsl, prm.maxstep) == (0.8, 1.25, 4.0, 1e-6, 5000)
        assert prm.rk_stages == 4 and prm.irs_eps == 0.8 and prm.irs_sweeps == 2
        with open(p, "w") as f:
            f.write("0.8 1.25\n")
        with pytest.raises(_lib.E2DError) as ei:
            e2d.read_input(p)
        assert ei.value.code == -2


def test_errors(lib):
    with pytest.raises(_lib.E2DError) as ei:
        e2d.Mesh.read("/nonexistent/mesh.dat")
    assert ei.value.code == -2
    x = np.array([0.0, 1.0, 0.0, 1.0])
    y = np.array([0.0, 0.0, 1.0, 1.0])
    cw = e2d.Mesh.from_arrays(x, y, np.array([[1, 3, 2]]))  # clockwise cell
    with pytest.raises(_lib.E2DError) as ei:
        cw.info()
    assert ei.value.code == -3 and "area" in str(ei.value)
    fan = e2d.Mesh.from_arrays(np.array([0.0, 1.0, 0.5, 0.5, 0.5]), np.array([0.0, 0.0, 1.0, -1.0, 2.0]),
                               np.array([[1, 2, 3], [2, 1, 4], [1, 2, 5]]))
    with pytest.raises(_lib.E2DError) as ei:
        fan.info()
    assert ei.value.code == -3
    bad = e2d.Mesh.from_arrays(x, y, np.array([[1, 2, 9]]))
    with pytest.raises(_lib.E2DError):
        bad.info()
    with pytest.raises(_lib.E2DError) as ei:
        e2d.Solver(e2d.Mesh.ogrid(16, 4), e2d.default_params(rk_stages=9))
    assert ei.value.code == -1


def test_binary_mesh_cache_roundtrip(lib, tmp_path):
    m = e2d.Mesh.ogrid(40, 10, seed=5)
    p = str(tmp_path / "m.bin")
    m.write(p, binary=True)
    assert os.path.getsize(p) == 16 + 16 * 40 * 11 + 12 * 800
    m2 = e2d.Mesh.read(p)
    for a, b in zip(m.nodes(), m2.nodes()):
        assert np.array_equal(a, b)
    with open(p, "rb") as f:
        head = f.read(os.path.getsize(p) - 4)
    with open(p, "wb") as f:
        f.write(head)
    with pytest.raises(_lib.E2DError, match="truncated"):
        e2d.Mesh.read(p)


def test_truncated_mesh_file(lib):
    with tempfile.TemporaryDirectory() as d:
        p = os.path.join(d, "m.dat")
        with open(p, "w") as f:
            f.write("4 2\n0 1 0 1\n0 0 1\n")
        with pytest.raises(_lib.E2DError) as ei:
            e2d.Mesh.read(p)
        assert ei.value.code == -2


@pytest.mark.parametrize("field,value,why", [
    ("gamma", 1.0, "gamma"), ("ma", float("nan"), "ma"), ("cfl", 0.0, "cfl"),
    ("epsl", float("nan"), "epsl"), ("maxstep", -1, "maxstep"), ("rk_stages", 0, "rk_stages"),
    ("rk_coef", [0.25, float("inf"), 0.5, 1.0], "rk_coef"), ("irs_sweeps", 17, "irs_sweeps"),
    ("irs_eps", -0.1, "irs_eps"), ("irs_eps", float("inf"), "irs_eps"), ("dt_cap", 0.0, "dt_cap"),
    ("entropy_eps", 0.0, "entropy_eps"), ("wall_box", -2.0, "wall_box"), ("precision", 2, "precision"),
    ("ordering", 3, "ordering"), ("block_size", 48, "block_size"), ("graph_iters", 300, "graph_iters"),
    ("limiter_freeze", -1, "limiter_freeze"), ("limiter", 4, "limiter"), ("limiter", -1, "limiter"),
    ("first_order_iters", -1, "first_order_iters"), ("positivity_fix", 2, "positivity_fix"), ("global_dt", 2, "global_dt"),
    ("far_field_fix", -1, "far_field_fix"),
])
def test_invalid_parameters_are_named(lib, field, value, why):
    """Every rejected parameter is reported by name, before any device work
    (so these run without a GPU)."""
    mesh = e2d.Mesh.ogrid(16, 4)
    with pytest.raises(_lib.E2DError) as ei:
        e2d.Solver(mesh, e2d.default_params(**{field: value}))
    assert ei.value.code == -1 and f"invalid parameters: {why}" in str(ei.value)
    with pytest.raises(_lib.E2DError) as ei:
        e2d.Batch([mesh, mesh], [e2d.default_params(), e2d.default_params(**{field: value})])
    assert ei.value.code == -1 and f"invalid parameters of case 1: {why}" in str(ei.value)


def test_smooth_limiter_needs_positive_k(lib):
    mesh = e2d.Mesh.ogrid(16, 4)
    with pytest.raises(_lib.E2DError, match="limiter_k"):
        e2d.Solver(mesh, e2d.default_params(limiter=1, limiter_k=0.0))


def test_valid_parameters_pass_validation(lib):
    """The reference defaults and the options at their documented values get
    past validation: without a GPU the failure is then the missing device."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("checks the no-device error path")
    mesh = e2d.Mesh.ogrid(16, 4)
    for kw in [{}, dict(precision=e2d.E2D_FP32, ordering=e2d.E2D_ORDER_RCM, limiter=1, limiter_k=10.0,
                        limiter_freeze_resd=1e-3, global_dt=1, far_field_fix=1, irs_eps=0.0, irs_sweeps=0)]:
        with pytest.raises(_lib.E2DError) as ei:
            e2d.Solver(mesh, e2d.default_params(**kw))
        assert ei.value.code != -1, str(ei.value)


def test_ogrid_geometry(lib):
    """NACA 0012 O-grid: wall nodes on the closed-trailing-edge thickness
    curve, far-field nodes on the circle of radius 20 about mid-chord, first
    radial spacing 2e-3 chord, geometric stretching (constant ratio of
    consecutive radial steps), and interior nodes moved by the jitter at most
    5 % of their smallest neighbour distance in each coordinate (wall and far
    field not moved)."""
    ni, nj = 128, 32
    x, y, _ = e2d.Mesh.ogrid(ni, nj, seed=3, jitter=0.0).nodes()
    X, Y = x.reshape(nj + 1, ni), y.reshape(nj + 1, ni)
    xw = X[0]
    thick = 0.6 * (0.2969 * np.sqrt(xw) - 0.1260 * xw - 0.3516 * xw ** 2 + 0.2843 * xw ** 3 - 0.1036 * xw ** 4)
    assert xw.min() >= 0.0 and xw.max() <= 1.0
    np.testing.assert_allclose(np.abs(Y[0]), np.where((np.arange(ni) == 0) | (2 * np.arange(ni) == ni), 0.0, thick),
                               atol=1e-15)
    np.testing.assert_allclose(np.hypot(X[nj] - 0.5, Y[nj]), 20.0, rtol=1e-12)
    step = np.hypot(np.diff(X, axis=0), np.diff(Y, axis=0))  # [nj, ni] radial steps
    assert np.all(np.abs(step[0] - 2e-3) < 0.05 * 2e-3), (step[0].min(), step[0].max())
    ratio = step[1:] / step[:-1]
    np.testing.assert_allclose(ratio, ratio[0, 0], rtol=1e-9)
    assert 1.0 < ratio[0, 0] < 1.5
    xj, yj, _ = e2d.Mesh.ogrid(ni, nj, seed=3, jitter=0.05).nodes()
    XJ, YJ = xj.reshape(nj + 1, ni), yj.reshape(nj + 1, ni)
    assert np.array_equal(XJ[[0, nj]], X[[0, nj]]) and np.array_equal(YJ[[0, nj]], Y[[0, nj]])
    # smallest distance to the four structured neighbours of each interior node
    h = np.full((nj - 1, ni), np.inf)
    for di, dj in [(1, 0), (-1, 0), (0, 1), (0, -1)]:
        xs = np.roll(X, -di, axis=1)[1 + dj:nj + dj]
        ys = np.roll(Y, -di, axis=1)[1 + dj:nj + dj]
        h = np.minimum(h, np.hypot(xs - X[1:nj], ys - Y[1:nj]))
    dx, dy = np.abs(XJ[1:nj] - X[1:nj]), np.abs(YJ[1:nj] - Y[1:nj])
    assert np.all(dx <= 0.05 * h * (1 + 1e-12)) and np.all(dy <= 0.05 * h * (1 + 1e-12))
    assert dx.max() > 0.02 * h[np.unravel_index(dx.argmax(), dx.shape)]  # the jitter is there


@pytest.mark.parametrize("kw,why", [
    (dict(precision=1), "only precision E2D_FP64"),
    (dict(limiter_freeze=3), "limiter_freeze and limiter_freeze_resd are not supported"),
    (dict(limiter_freeze_resd=1e-3), "limiter_freeze and limiter_freeze_resd are not supported"),
    (dict(cfl=0.0), "invalid parameters: cfl"),
])
def test_step_noalloc_refuses_options_it_does_not_carry(lib, kw, why):
    """The allocation-free entry point refuses, by name and before touching
    any pointer or device, the options that it cannot honour (FP32 stencil,
    limiter freezing) instead of ignoring them; the pointers here are never
    dereferenced."""
    import ctypes
    p = e2d.default_params(**kw)
    fake = ctypes.c_void_p(1 << 20)  # non-null and aligned; refused before any use
    epsm = ctypes.c_double(0.0)
    rc = lib.e2d_step_noalloc(64, fake, fake, fake, fake, ctypes.byref(p), 1, fake, fake, ctypes.byref(epsm), None)
    assert rc == -1 and why in lib.e2d_last_error().decode()


def test_step_noalloc_names_every_alignment(lib):
    import ctypes
    p = e2d.default_params()
    ok, odd = ctypes.c_void_p(1 << 20), ctypes.c_void_p((1 << 20) + 4)
    epsm = ctypes.c_double(0.0)
    rc = lib.e2d_step_noalloc(64, ok, ok, ok, odd, ctypes.byref(p), 1, ok, ok, ctypes.byref(epsm), None)
    msg = lib.e2d_last_error().decode()
    assert rc == -1 and "area and resid 8-byte aligned" in msg


@pytest.mark.parametrize("ni,nj,seed,jitter", [(8, 1, 1, 0.05), (64, 16, 5, 0.05), (128, 32, 1, 0.05),
                                               (256, 64, 9, 0.0), (512, 128, 1, 0.05), (2048, 1024, 1, 0.05)])
def test_oracle_ogrid_equals_library_ogrid(lib, oracle, ni, nj, seed, jitter):
    """The oracle's statement of the O-grid generator (used by the CPU arm of
    the benchmark, which must not load the product library) makes the same
    mesh bit for bit, up to the large-mesh configuration's 2048 x 1024."""
    a = e2d.Mesh.ogrid(ni, nj, seed=seed, jitter=jitter).nodes()
    b = oracle.ogrid(ni, nj, seed=seed, jitter=jitter)
    for u, v in zip(a, b):
        assert np.array_equal(np.asarray(u).ravel(), np.asarray(v).ravel())

"""e2d_step_noalloc: iterations for callers that may not allocate device memory.

Such a caller (for example a plug-in whose host application owns every device
allocation) holds the mesh layout and the state in buffers it was given, and
the library keeps its working arrays in a fixed device array instead of
allocating.  This test hands the entry point buffers allocated here (the test
itself may allocate), calls it twice in a row and checks both calls against the
regular allocating path, e2d_step, through the C ABI: the FP64 state and the
residual history must be identical bit for bit, as in the other FP64 parity
tests.  It lives in a file of its own that pytest collects last.
"""
import ctypes

import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d
from gpueularsolver2d_gb300 import _lib

pytestmark = pytest.mark.gpu


def file_order_layout(mesh):
    """The solver's cell-local layout in file order, built from the reference
    numbering that e2d_mesh_topology exports (include/euler2d.h)."""
    ei, ed, ci, cd = mesh.topology()
    x, y, tri = mesh.nodes()
    n = ci.shape[0]
    celledge, neicell = ci[:, 1:4], ci[:, 4:7]
    topo = np.zeros((n, 4), np.int32)
    S = np.zeros((3, n, 2))
    R = np.zeros((3, n, 2))
    cells = np.arange(1, n + 1)
    for k in range(3):
        n1 = tri[:, (k + 1) % 3] - 1
        n2 = tri[:, (k + 2) % 3] - 1
        S[k, :, 0] = y[n2] - y[n1]  # vectory
        S[k, :, 1] = x[n1] - x[n2]  # vectorx
        e = celledge[:, k] - 1
        R[k, :, 0] = ed[e, 3] - cd[:, 1]
        R[k, :, 1] = ed[e, 4] - cd[:, 2]
        nb = neicell[:, k]
        inner = nb > 0
        right = (ei[e, 2] == cells).astype(np.int32)
        slot = np.argmax(celledge[np.where(inner, nb - 1, 0)] == (e + 1)[:, None], axis=1)
        topo[:, k] = np.where(inner, ((nb - 1) << 3) | (right << 2) | slot, nb)
    topo[:, 3] = ci[:, 0]
    return topo.ravel(), S.ravel(), R.ravel(), cd[:, 0].copy()


def test_step_noalloc_matches_step(lib):
    import torch
    mesh = e2d.Mesh.ogrid(48, 12, seed=6)
    p = e2d.default_params(ma=0.6, alpha_deg=1.5, cfl=1.5, ordering=e2d.E2D_ORDER_FILE)
    ref = e2d.Solver(mesh, p)
    topo, S, R, area = file_order_layout(mesh)
    dev = torch.device("cuda", torch.cuda.current_device())
    t_topo = torch.from_numpy(topo).to(dev)
    t_S = torch.from_numpy(S).to(dev)
    t_R = torch.from_numpy(R).to(dev)
    t_area = torch.from_numpy(area).to(dev)
    t_w = torch.from_numpy(ref.state().ravel().copy()).to(dev)
    n = ref.ncell
    epsm = ctypes.c_double(0.0)
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    for calls, iters in enumerate((3, 4)):
        t_res = torch.zeros(iters, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        rc = lib.e2d_step_noalloc(n, ptr(t_topo), ptr(t_S), ptr(t_R), ptr(t_area), ctypes.byref(p), iters,
                                  ptr(t_w), ptr(t_res), ctypes.byref(epsm), None)
        _lib.check(rc)
        ref.step(iters)
        w = t_w.cpu().numpy().reshape(n, 4)
        assert np.array_equal(w, ref.state()), f"call {calls + 1}: {np.max(np.abs(w - ref.state()))}"
        assert np.array_equal(t_res.cpu().numpy(), ref.history()[-iters:]), f"call {calls + 1}"
    assert epsm.value == ref.residual_norm()


def test_step_noalloc_rejects_too_many_cells(lib):
    import torch
    buf = torch.zeros(64, dtype=torch.float64, device="cuda")
    p = e2d.default_params()
    epsm = ctypes.c_double(0.0)
    ptr = ctypes.c_void_p(buf.data_ptr())
    rc = lib.e2d_step_noalloc(32769, ptr, ptr, ptr, ptr, ctypes.byref(p), 1, ptr, ptr, ctypes.byref(epsm),
                              None)
    assert rc == -6
    assert "32768" in lib.e2d_last_error().decode()


def test_step_noalloc_refuses_out_of_range_topology(lib):
    """A face code that names a cell outside the mesh (or a slot above 2, or a
    negative code other than -1 / -2) is caught on the GPU before any pass
    gathers through it: the call returns E2D_ERR_ARG, the state and the
    residual buffer are untouched, and the next valid call works."""
    import torch
    mesh = e2d.Mesh.ogrid(48, 12, seed=6)
    p = e2d.default_params(ma=0.6, alpha_deg=1.5, cfl=1.5, ordering=e2d.E2D_ORDER_FILE)
    ref = e2d.Solver(mesh, p)
    topo, S, R, area = file_order_layout(mesh)
    n = ref.ncell
    dev = torch.device("cuda", torch.cuda.current_device())
    t_S, t_R, t_area = (torch.from_numpy(a).to(dev) for a in (S, R, area))
    w0 = ref.state().ravel().copy()
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    t4 = topo.reshape(n, 4)
    i = int(np.flatnonzero(t4[:, 0] >= 0)[0])
    for bad_code in ((n + 3) << 3 | (int(t4[i, 0]) & 7), (int(t4[i, 0]) & ~3) | 3, -5):
        bad = t4.copy()
        bad[i, 0] = bad_code
        t_topo = torch.from_numpy(bad.ravel().copy()).to(dev)
        t_w = torch.from_numpy(w0).to(dev)
        t_res = torch.full((2,), -7.0, dtype=torch.float64, device=dev)
        epsm = ctypes.c_double(0.0)
        rc = lib.e2d_step_noalloc(n, ptr(t_topo), ptr(t_S), ptr(t_R), ptr(t_area), ctypes.byref(p), 2, ptr(t_w),
                                  ptr(t_res), ctypes.byref(epsm), None)
        assert rc == -1 and "out of range" in lib.e2d_last_error().decode(), bad_code
        assert np.array_equal(t_w.cpu().numpy(), w0) and np.all(t_res.cpu().numpy() == -7.0)
    t_topo = torch.from_numpy(topo).to(dev)
    t_w = torch.from_numpy(w0).to(dev)
    t_res = torch.zeros(2, dtype=torch.float64, device=dev)
    epsm = ctypes.c_double(0.0)
    _lib.check(lib.e2d_step_noalloc(n, ptr(t_topo), ptr(t_S), ptr(t_R), ptr(t_area), ctypes.byref(p), 2, ptr(t_w),
                                    ptr(t_res), ctypes.byref(epsm), None))
    ref.step(2)
    assert np.array_equal(t_w.cpu().numpy().reshape(n, 4), ref.state())

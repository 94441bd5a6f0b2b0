"""The solver keeps its topology array in a persisting L2 carve-out, a limit
of the process's CUDA context.  While a solver exists the limit is raised;
once the last solver (or batch) is destroyed the limit is back at its
previous value, so later work in the process gets the whole L2."""
import ctypes

import pytest

import gpueularsolver2d_gb300 as e2d

pytestmark = pytest.mark.gpu

CU_LIMIT_PERSISTING_L2_CACHE_SIZE = 0x06


def test_persisting_l2_limit_is_restored(lib):
    import torch
    torch.cuda.synchronize()  # the primary context, current in this thread
    cuda = ctypes.CDLL("libcuda.so.1")

    def limit():
        v = ctypes.c_size_t(0)
        assert cuda.cuCtxGetLimit(ctypes.byref(v), CU_LIMIT_PERSISTING_L2_CACHE_SIZE) == 0
        return v.value

    before = limit()
    mesh = e2d.Mesh.ogrid(256, 64, seed=2)
    a = e2d.Solver(mesh, e2d.default_params(precision=e2d.E2D_FP32))
    b = e2d.Solver(mesh, e2d.default_params(precision=e2d.E2D_FP32))
    a.step(2)
    b.step(2)
    during = limit()
    assert during >= before
    a.close()
    assert limit() == during  # b still uses it
    b.close()
    assert limit() == before

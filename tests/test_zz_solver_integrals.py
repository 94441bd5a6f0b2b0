"""The solver-level FP64 integrals (e2d_solver_integrals) on the GPU."""
import pytest

import gpueularsolver2d_gb300 as e2d

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", [e2d.E2D_FP64, e2d.E2D_FP32])
def test_solver_integrals_match_the_host_function(lib, precision):
    """e2d_solver_integrals of a solver's state equals e2d_state_integrals of
    the same state read back (one layout, one summation order)."""
    mesh = e2d.Mesh.ogrid(48, 12, seed=3)
    p = e2d.default_params(ma=0.5, alpha_deg=1.25, cfl=1.5, precision=precision,
                           ordering=e2d.E2D_ORDER_MORTON)
    s = e2d.Solver(mesh, p)
    s.step(50)
    a = s.integrals()
    b = e2d.state_integrals(mesh, p, s.state())
    for k in a:
        assert a[k] == pytest.approx(b[k], rel=1e-12, abs=1e-15), k
    cl, cd = s.forces()
    assert a["cl"] == cl and a["cd"] == cd

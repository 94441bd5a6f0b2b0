"""Unusable states come back as error codes from the host, without faulting
the GPU: a state with a NaN or a non-positive density is flagged by the last
stage's physicality check of the first iteration (E2D_ERR_DIVERGED, -5), and
the solver stays usable: a good state set afterwards steps normally."""
import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d
from gpueularsolver2d_gb300._lib import E2DError

pytestmark = pytest.mark.gpu

DIVERGED = -5  # E2D_ERR_DIVERGED in include/euler2d.h


@pytest.mark.parametrize("precision", [e2d.E2D_FP64, e2d.E2D_FP32])
@pytest.mark.parametrize("bad_value", [float("nan"), -0.5])
def test_bad_state_is_reported_and_the_solver_recovers(lib, precision, bad_value):
    mesh = e2d.Mesh.ogrid(32, 8, seed=2)
    s = e2d.Solver(mesh, e2d.default_params(ma=0.5, alpha_deg=1.0, precision=precision))
    good = s.state()
    w = good.copy()
    w[17, 0] = bad_value  # density of one cell
    s.set_state(w)
    with pytest.raises(E2DError) as ei:
        s.step(1)
    assert ei.value.code == DIVERGED and "diverged" in str(ei.value)
    s.set_state(good)
    s.step(3)
    assert np.all(np.isfinite(s.state())) and np.all(s.state()[:, 0] > 0)


"""FP64 integrals of a state (e2d_state_integrals, no GPU) against the CPU
oracle on a non-steady state: the boundary mass fluxes are the oracle's
first-order boundary-edge fluxes summed by kind (the slip wall's is zero to
rounding), their sum is the oracle's
mass residual summed over the cells (interior faces cancel), the mass is the
area-weighted density sum, and lift and drag are the wall-pressure integral.
Tolerances: 1e-12 relative for sums taken in a different order, 1e-11 of
the summed boundary flux magnitudes for the residual identity."""
import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d

K_PI = 3.14159265358979  # the free stream's pi (gpu_init.cu)


@pytest.mark.parametrize("ni,nj,seed,ma,alpha,ordering", [
    (48, 12, 3, 0.5, 1.25, e2d.E2D_ORDER_FILE),
    (64, 16, 7, 0.7, 2.5, e2d.E2D_ORDER_MORTON),
])
def test_integrals_match_the_oracle(lib, oracle, ni, nj, seed, ma, alpha, ordering):
    mesh = e2d.Mesh.ogrid(ni, nj, seed=seed)
    p = e2d.default_params(ma=ma, alpha_deg=alpha, cfl=1.5, ordering=ordering)
    x, y, tri = mesh.nodes()
    case = oracle.Case(x, y, tri, oracle.params_from_e2d(p))
    case.run(300)
    w = case.state()
    got = e2d.state_integrals(mesh, p, w)

    ei, ed, ci, cd = case.topology()
    probe = case.stage_probe()
    flux = probe["flux"][:, 0]  # mass flux times the face length of each edge, from its left cell
    far, wall = ei[:, 0] == 1, ei[:, 0] == 2
    assert far.sum() == ni and wall.sum() == ni
    scale = np.abs(flux[far | wall]).sum()
    assert got["mass_flux_far"] == pytest.approx(flux[far].sum(), rel=1e-12, abs=1e-15 * scale)
    assert got["mass_flux_wall"] == pytest.approx(flux[wall].sum(), rel=1e-12, abs=1e-15 * scale)
    net = probe["res"][:, 0].sum()  # interior faces cancel in the cell residuals
    assert abs(got["mass_flux_far"] + got["mass_flux_wall"] - net) < 1e-11 * scale
    # 300 iterations in, the start-up transient is crossing the far field
    # (each far-field face carries O(1)); the slip wall passes no mass
    assert abs(got["mass_flux_far"]) > 1e-4
    assert abs(got["mass_flux_wall"]) < 1e-12

    assert got["mass"] == pytest.approx(float(np.sum(w[:, 0] * cd[:, 0])), rel=1e-12)

    # lift and drag: wall pressure of the wall cells against p_inf on the wall faces
    left = ei[wall, 1] - 1
    u = w[left]
    pres = (p.gamma - 1.0) * (u[:, 3] - 0.5 * (u[:, 1] ** 2 + u[:, 2] ** 2) / u[:, 0])
    vx, vy = ed[wall, 1], ed[wall, 2]
    fx = np.sum((pres - case.pis()) * vy)
    fy = np.sum((pres - case.pis()) * vx)
    a = alpha * K_PI / 180.0
    assert got["cd"] == pytest.approx((fx * np.cos(a) + fy * np.sin(a)) / 0.5, rel=1e-11, abs=1e-14)
    assert got["cl"] == pytest.approx((-fx * np.sin(a) + fy * np.cos(a)) / 0.5, rel=1e-11, abs=1e-14)


def test_integrals_of_the_free_stream(lib):
    """The free stream at zero incidence on the whole mesh: the mass is the
    total area (unit density) and the symmetric profile carries no lift."""
    mesh = e2d.Mesh.ogrid(32, 8, seed=1)
    p = e2d.default_params(ma=0.5, alpha_deg=0.0)
    n = mesh.info().ncell
    from gpueularsolver2d_gb300.warmstart import freestream
    w = freestream(0.5, 0.0, n)
    got = e2d.state_integrals(mesh, p, w)
    _, _, _, cd = mesh.topology()
    assert got["mass"] == pytest.approx(float(cd[:, 0].sum()), rel=1e-12)
    assert abs(got["cl"]) < 1e-12


def test_integrals_reject_bad_input(lib):
    mesh = e2d.Mesh.ogrid(16, 4)
    with pytest.raises(ValueError):
        e2d.state_integrals(mesh, e2d.default_params(), np.zeros((5, 4)))
    with pytest.raises(Exception, match="entropy_eps"):
        e2d.state_integrals(mesh, e2d.default_params(entropy_eps=0.0), np.ones((128, 4)))

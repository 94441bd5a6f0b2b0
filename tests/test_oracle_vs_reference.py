"""Pin the CPU oracle to the reference's own code.

Two sources, both the reference's functions, never the oracle itself:
* tests/golden/ogrid24x6_seed3.npz, written by tests/golden/make_golden.py
  from the reference harness (always available);
* the reference harness itself, built in place from the reference sources
  when they are present (skipped otherwise).

Integer set-up (edge numbering, left/right cells, boundary tags, neighbour
tables) and the set-up geometry must match bit for bit.  The stage quantities
come from the reference's host scheme functions (gpu_solver.cu:1043-1503),
which differ from its GPU kernels -- and so from the oracle, which follows the
kernels -- only in rounding: the host Gradient multiplies by n*|S| instead of
S (1273-1286), the host Roe flux uses sqrt(rL*rR) (1393) and divides where the
kernel multiplies by a reciprocal (1065-1071).  Those are compared to 1e-12
relative to each array's scale.
"""
import os
import tempfile

import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d
from conftest import reference_mesh

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "ogrid24x6_seed3.npz")


def _input_params(oracle, line):
    v = line.split()
    return oracle.params(ma=float(v[0]), alpha_deg=float(v[1]), gamma=float(v[2]), pin=float(v[3]),
                         tin=float(v[4]), cfl=float(v[5]), epsl=float(v[6]), maxstep=int(v[7]))


def _rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def check_setup(case, ref):
    ei, ed, ci, cd = case.topology()
    assert list(ref["counts"]) == [case.ncell, case.nnode, case.nedge, case.nwall, case.nfar]
    assert np.array_equal(ei.ravel(), ref["edge_i"])
    assert np.array_equal(ed.ravel(), ref["edge_d"])
    assert np.array_equal(ci.ravel(), ref["cell_i"])
    assert np.array_equal(cd.ravel(), ref["cell_d"])
    assert np.array_equal(case.state(), ref["w_init"].reshape(-1, 7)[:, :4])
    assert case.pis() == ref["pis"][0]


def check_stage(case, ref):
    ei, ed, ci, cd = case.topology()
    pr = case.stage_probe()
    assert np.array_equal(pr["umm"].ravel(), ref["umm"])
    assert _rel(pr["ghost"].ravel(), ref["ghost"]) < 1e-12
    assert _rel(pr["grad"].ravel(), ref["grad"]) < 1e-12
    flux_ref = ref["flux_raw"].reshape(-1, 4) * ed[:, :1]  # kernel_Flux2 multiplies by vectorn
    assert _rel(pr["flux"], flux_ref) < 1e-12
    # the host Flux adds each face's spectral radius into its cells
    sr_sum = pr["sr"][ci[:, 1:4] - 1].sum(axis=1)
    assert _rel(sr_sum, ref["sr_sum"]) < 1e-12


def test_golden_setup_and_stage(oracle):
    g = np.load(GOLDEN)
    p = _input_params(oracle, str(g["input"]))
    case = oracle.Case(g["x"], g["y"], g["tri"], p)
    check_setup(case, g)
    case.set_state(g["w_in"])
    check_stage(case, g)


def test_golden_mesh_is_the_generator_output(lib):
    g = np.load(GOLDEN)
    x, y, tri = e2d.Mesh.ogrid(24, 6, seed=3).nodes()
    assert np.array_equal(x, g["x"]) and np.array_equal(y, g["y"]) and np.array_equal(tri, g["tri"])


@pytest.mark.parametrize("name", ["2822-3k.dat", "2822-1w.dat"])
def test_live_reference_setup_on_fixture_meshes(oracle, name):
    path = reference_mesh(name)
    if path is None or oracle.ref_harness_path() is None:
        pytest.skip("reference checkout not available")
    line = "0.7 1.25 1.4 101325 288.15 2.0 1e-6 10"
    ref = oracle.run_reference("geo", path, line)
    check_setup(oracle.Case.from_file(path, _input_params(oracle, line)), ref)


@pytest.mark.parametrize("ni,nj,seed,line", [
    (40, 10, 1, "0.5 1.25 1.4 101325 288.15 2.0 1e-6 10"),
    (64, 16, 9, "0.8 -1.0 1.4 90000 250.0 1.2 1e-6 10"),
])
def test_live_reference_stage_nonuniform(lib, oracle, ni, nj, seed, line):
    if oracle.ref_harness_path() is None:
        pytest.skip("reference checkout not available")
    mesh = e2d.Mesh.ogrid(ni, nj, seed=seed)
    x, y, tri = mesh.nodes()
    case = oracle.Case(x, y, tri, _input_params(oracle, line))
    case.run(20)
    w = case.state()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "m.dat")
        mesh.write(path)
        ref = oracle.run_reference("stage", path, line, w_in=w)
    fresh = oracle.Case(x, y, tri, _input_params(oracle, line))
    check_setup(fresh, ref)
    fresh.set_state(w)
    check_stage(fresh, ref)

"""The reference's function surface (libeuler2d_compat.a, include/euler2d_compat.h).

CPU: inputMesh / Initialization / CalculationMeshGeo through the compat layer
must produce exactly what the reference's own functions produce (edge table in
discovery order, neighbours, CLog, areas, centres, WallEdge list, wall-node
flags, free-stream state, PIS).

GPU: the reference's own main() (gpu_fvm.cu) linked against the compat layer
runs the GB300 solver and prints the same residual history, bit for bit, as
the C ABI's FP64 solve; its output files describe the converged field.
"""
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

import gpueularsolver2d_gb300 as e2d
from gpueularsolver2d_gb300 import build as pkg_build
from conftest import ROOT, reference_mesh

CUDA_LIB = "/usr/local/cuda/lib64"
INPUT = "0.6 1.5 1.4 101325 288.15 1.5 1e-9 30"


def _driver(tmp):
    exe = os.path.join(tmp, "compat_driver")
    subprocess.run(["g++", "-O2", "-std=c++17", f"-I{os.path.join(ROOT, 'include')}",
                    os.path.join(ROOT, "tests", "compat_driver.cpp"), pkg_build.COMPAT,
                    f"-L{pkg_build.LIBDIR}", "-leuler2d", f"-L{CUDA_LIB}", "-lcudart",
                    f"-Wl,-rpath,{pkg_build.LIBDIR}", "-o", exe], check=True)
    return exe


def _dumps(d):
    out = {}
    for name, dt in [("counts", np.int32), ("edge_i", np.int32), ("edge_d", np.float64), ("cell_i", np.int32),
                     ("cell_d", np.float64), ("w_init", np.float64), ("pis", np.float64), ("wall_i", np.int32),
                     ("nlog", np.int32)]:
        out[name] = np.fromfile(os.path.join(d, name + ".bin"), dt)
    return out


def _meshes():
    items = []
    p = reference_mesh("2822-3k.dat")
    if p:
        items.append(("rae2822_3k", p))
    return items


@pytest.mark.parametrize("which", ["ogrid", "rae2822_3k"])
def test_compat_setup_matches_reference(lib, oracle, which):
    if oracle.ref_harness_path() is None:
        pytest.skip("reference sources not available")
    with tempfile.TemporaryDirectory() as d:
        if which == "ogrid":
            mesh_path = os.path.join(d, "src.dat")
            e2d.Mesh.ogrid(40, 10, seed=4).write(mesh_path)
        else:
            mesh_path = reference_mesh("2822-3k.dat")
            if mesh_path is None:
                pytest.skip("reference meshes not available")
        ref = oracle.run_reference("geo0", mesh_path, INPUT)
        run = os.path.join(d, "run")
        os.makedirs(run)
        shutil.copyfile(mesh_path, os.path.join(run, "2822-3k.dat"))
        with open(os.path.join(run, "input.dat"), "w") as f:
            f.write(INPUT + "\n")
        res = subprocess.run([_driver(d)], cwd=run, capture_output=True, text=True)
        assert res.returncode == 0, res.stdout + res.stderr
        assert "inputData finished!" in res.stdout
        got = _dumps(run)
    for k, v in got.items():
        assert np.array_equal(v, ref[k]), k


def test_compat_missing_mesh_exits_like_reference(lib):
    with tempfile.TemporaryDirectory() as d:
        res = subprocess.run([_driver(d)], cwd=d, capture_output=True, text=True)
        assert res.returncode == 0 and "Cannot open the mesh data file!" in res.stdout


@pytest.mark.gpu
def test_reference_main_runs_on_gb300_solver(lib):
    import build_ref  # oracle/build_ref.py
    src = build_ref.source_dir()
    if src is None:
        pytest.skip("reference sources not available")
    mesh = e2d.Mesh.ogrid(48, 12, seed=8)
    with tempfile.TemporaryDirectory() as d:
        exe = os.path.join(d, "ref_main_on_e2d")
        subprocess.run(["nvcc", "-gencode", "arch=compute_103a,code=sm_103a", "-w", f"-I{src}",
                        os.path.join(src, "gpu_fvm.cu"), pkg_build.COMPAT, f"-L{pkg_build.LIBDIR}", "-leuler2d",
                        f"-Xlinker", f"-rpath={pkg_build.LIBDIR}", "-o", exe], check=True)
        mesh.write(os.path.join(d, "2822-3k.dat"))
        with open(os.path.join(d, "input.dat"), "w") as f:
            f.write(INPUT + "\n")
        res = subprocess.run([exe], cwd=d, capture_output=True, text=True, timeout=300)
        assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
        assert "All Computation's Finished!!" in res.stdout
        lines = [l for l in res.stdout.splitlines() if l.count(",") == 1 and l.split(",")[0].isdigit()]
        resid = np.array([float(l.split(",")[1]) for l in lines])
        assert len(resid) == 30
        p = e2d.default_params(ma=0.6, alpha_deg=1.5, cfl=1.5, ordering=e2d.E2D_ORDER_MORTON)
        s = e2d.Solver(mesh, p)
        hist = s.solve(30, 1e-9)
        np.testing.assert_allclose(resid, hist, rtol=1e-15)
        # the field written by the reference's Output() is the converged one
        vals = np.loadtxt(os.path.join(d, "unresult.plt"), skiprows=6, max_rows=mesh.info().nnode)
        assert np.std(vals[:, 2]) > 1e-4  # density varies over the nodes
        # content parity of the writers: the e2d_solve command on the same files
        # writes unresult.plt and unairfoilpress.plt equal to what the
        # reference's own Node_Computing / Output (gpu_fvm.cu:71-195) write from
        # the same state, value for value at the printed precision
        d2 = os.path.join(d, "cli")
        os.makedirs(d2)
        mesh.write(os.path.join(d2, "2822-3k.dat"))
        with open(os.path.join(d2, "input.dat"), "w") as f:
            f.write(INPUT + "\n")
        res2 = subprocess.run([pkg_build.CLI], cwd=d2, capture_output=True, text=True, timeout=300)
        assert res2.returncode == 0, res2.stdout[-2000:] + res2.stderr[-2000:]
        for name in ("unresult.plt", "unairfoilpress.plt"):
            ref_txt = open(os.path.join(d, name)).read().splitlines()
            cli_txt = open(os.path.join(d2, name)).read().splitlines()
            assert len(ref_txt) == len(cli_txt), name
            hdr = 6 if name == "unresult.plt" else 3
            assert ref_txt[:hdr] == cli_txt[:hdr], name
            a = np.array([[float(v) for v in l.split()] for l in ref_txt[hdr:]], dtype=object)
            b = np.array([[float(v) for v in l.split()] for l in cli_txt[hdr:]], dtype=object)
            for ra, rb in zip(a, b):
                np.testing.assert_allclose(np.array(rb, float), np.array(ra, float), rtol=0, atol=2e-10,
                                           err_msg=name)
            differing = sum(x != y for x, y in zip(ref_txt, cli_txt))
            print(f"{name}: {len(ref_txt)} lines, {differing} differ in text (last printed digit)")


@pytest.mark.gpu
def test_cli_reproduces_reference_files(lib):
    mesh = e2d.Mesh.ogrid(48, 12, seed=8)
    with tempfile.TemporaryDirectory() as d:
        mesh.write(os.path.join(d, "2822-3k.dat"))
        with open(os.path.join(d, "input.dat"), "w") as f:
            f.write("0.6 1.5 1.4 101325 288.15 1.5 1e-9 250\n")
        res = subprocess.run([pkg_build.CLI], cwd=d, capture_output=True, text=True, timeout=300)
        assert res.returncode == 0, res.stdout[-2000:] + res.stderr[-2000:]
        lines = [l for l in res.stdout.splitlines() if l.count(",") == 1 and l.split(",")[0].isdigit()]
        assert len(lines) == 250 and lines[0].startswith("1,")
        for name in ("unresult.plt", "unresidual.plt", "unairfoilpress.plt"):
            assert os.path.getsize(os.path.join(d, name)) > 0
        txt = open(os.path.join(d, "unresidual.plt")).read().splitlines()
        assert txt[2].startswith("ZONE I=250 J=1") and len(txt) == 3 + 2  # every 100th step
        cp = open(os.path.join(d, "unairfoilpress.plt")).read().splitlines()
        assert cp[2].startswith("ZONE N=96 E=48")

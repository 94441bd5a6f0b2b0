"""Generate golden vectors from the reference's OWN code (oracle/_ref).

Runs the reference harness (the reference's gpu_init.cu / gpu_solver.cu host
functions, compiled in place by oracle/build_ref.py) on a small seeded
NACA 0012 O-grid and stores its outputs:

* set-up (CalculationMeshGeo + changeEdge): edge and cell tables, areas,
  centroids, the free-stream state and PIS;
* one stage of the reference's host scheme functions (Boundary, Gradient,
  per-edge Flux) on a non-uniform state -- the CPU oracle's state after 15
  iterations, stored alongside as the input.

Usage: python tests/golden/make_golden.py   (needs the reference checkout)
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import gpueularsolver2d_gb300 as e2d  # noqa: E402
import pyoracle  # noqa: E402

INPUT = "0.6 2.0 1.4 101325 288.15 1.5 1e-6 100"


def main():
    mesh = e2d.Mesh.ogrid(24, 6, seed=3)
    x, y, tri = mesh.nodes()
    p = pyoracle.params(ma=0.6, alpha_deg=2.0, cfl=1.5)
    case = pyoracle.Case(x, y, tri, p)
    case.run(15)
    w_in = case.state()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "m.dat")
        mesh.write(path)
        out = pyoracle.run_reference("stage", path, INPUT, w_in=w_in)
    keep = {k: v for k, v in out.items() if k != "stdout"}
    np.savez_compressed(os.path.join(HERE, "ogrid24x6_seed3.npz"), x=x, y=y, tri=tri, w_in=w_in,
                        input=np.array(INPUT), **keep)
    print("wrote", os.path.join(HERE, "ogrid24x6_seed3.npz"), sorted(keep))


if __name__ == "__main__":
    main()

"""One case run to a residual drop with explicitly flagged scheme options.

The reference scheme (per-face limiter, gpu_solver.cu:456-549) does not reach
a 1e-6 drop on the transonic O-grid cases: at M 0.80 on the 512 x 128 mesh it
diverges after about 4.6k (CFL 2) to 9.4k (CFL 1) iterations whatever the
entropy fix, smoothing or per-face limiter form, while the first-order scheme
converges.  This driver runs a case with the options that make it converge,
every one named on the command line and in the result:

* a cell-wise limiter (``--limiter 3``: per cell and component the smallest
  Venkatakrishnan value over the cell's interior faces; ``2`` is the
  Barth-Jespersen form of the reference's values);
* the limiter values frozen once Resd falls to ``--freeze`` (or at iteration
  ``--freeze-after``, whichever comes first: on finer meshes the residual
  can level off just above the freeze level);
* the FP32 stencil down to ``--switch``, then a new FP64 solver from the state
  reached, its limiter values frozen after its first iteration, to
  ``--target`` (FP32 states stall near 1e-5).

Run ``python -m gpueularsolver2d_gb300.converge --help``; the result is one
JSON object (iterations, wall time of each phase, the drop reached, CL/CD).
"""
from __future__ import annotations

import argparse
import json
import sys
import time

from . import api as e2d
from .warmstart import SolverSettings, run_to_drop


def settings_from(args) -> SolverSettings:
    return SolverSettings(cfl=args.cfl, freeze=args.freeze_after, freeze_resd=args.freeze, precision=e2d.E2D_FP32,
                          limiter=args.limiter,
                          limiter_k=args.limiter_k, refreeze_resd=args.switch, tail_precision=e2d.E2D_FP64,
                          irs_eps=args.irs_eps, positivity_fix=args.positivity_fix,
                          first_order_iters=args.first_order_iters)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--ni", type=int, default=512)
    ap.add_argument("--nj", type=int, default=128)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--mach", type=float, default=0.80)
    ap.add_argument("--alpha", type=float, default=1.25)
    ap.add_argument("--cfl", type=float, default=2.0)
    ap.add_argument("--irs-eps", type=float, default=0.6)
    ap.add_argument("--limiter", type=int, default=3)
    ap.add_argument("--limiter-k", type=float, default=5.0)
    ap.add_argument("--freeze", type=float, default=3e-3, help="freeze the limiter values at this Resd")
    ap.add_argument("--freeze-after", type=int, default=0,
                    help="freeze the limiter values at this iteration if Resd has not reached --freeze (0: never)")
    ap.add_argument("--switch", type=float, default=2e-5, help="FP32 down to this Resd, then FP64")
    ap.add_argument("--target", type=float, default=1e-6)
    ap.add_argument("--maxit", type=int, default=400000)
    ap.add_argument("--positivity-fix", type=int, default=0)
    ap.add_argument("--first-order-iters", type=int, default=0)
    ap.add_argument("--json", default=None)
    args = ap.parse_args(argv)
    t0 = time.perf_counter()
    mesh = e2d.Mesh.ogrid(args.ni, args.nj, seed=args.seed)
    st = settings_from(args)
    out = run_to_drop(mesh, args.mach, args.alpha, st, args.target, args.maxit)
    out["settings"] = {k: getattr(st, k) for k in st.__dataclass_fields__}
    out["case"] = {"mesh": f"NACA0012 O-grid {args.ni}x{args.nj} seed {args.seed}", "cells": 2 * args.ni * args.nj,
                   "mach": args.mach, "alpha": args.alpha}
    out["command"] = "python -m gpueularsolver2d_gb300.converge " + " ".join(sys.argv[1:] if argv is None else argv)
    out["total_s"] = time.perf_counter() - t0
    txt = json.dumps(out, indent=1)
    print(txt)
    if args.json:
        with open(args.json, "w") as f:
            f.write(txt)
    return out


if __name__ == "__main__":
    main()

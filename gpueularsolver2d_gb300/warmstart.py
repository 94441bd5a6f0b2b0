"""Learned warm start: a coordinate MLP trained on steady solutions of the
solver predicts the initial conserved field of a new flow condition.

Pipeline (no reference counterpart; the plain solver stays the oracle):

1. ``generate``: steady solutions for sampled (Mach, alpha) on one mesh,
   computed by the batched solver (FP32 stencil) with the limiter-freeze
   option, the same settings for every case.
2. ``Dataset``: per-cell features (x, y, log wall distance, Mach, sin a, cos a,
   16 random Fourier features of (x, y); e2d_mlp_features) normalised to zero
   mean / unit variance for the first six, and targets W - W_inf(M, a) scaled
   per component.
3. ``train``: Adam on random batches, all on the GPU (e2d_mlp_train), the
   step size decaying on a cosine (e2d_mlp_set_lr between chunks of steps).
4. ``predict``: W_inf + scale * MLP(features) for a new condition.
5. ``evaluate``: for held-out conditions, iterations and wall time to the
   target drop from the free stream and from the prediction, with the same
   solver settings and the same residual normalisation (the free-stream run's
   first-iteration density change), and the converged CL / CD of both.  Both
   runs freeze the limiter values at Resd 1e-3 and again from the state at
   1e-5 (``refreeze_resd``): a warm run reaches 1e-3 within a few hundred
   iterations, on a state that still carries the prediction's error, and
   values frozen there would keep that error in the converged lift.  The free
   stream is the fallback (``run_warm``): a prediction that is not physical in
   every cell is not used, and a warm run that diverges is run again from the
   free stream, with the failed attempt's cost counted.

Run ``python -m gpueularsolver2d_gb300.warmstart --help``.
"""
from __future__ import annotations

import argparse
import json
import math
import sys
import time
from dataclasses import dataclass

import numpy as np

from . import api as e2d
from ._lib import E2DError

GAMMA = 1.4


def conditions(n: int, seed: int, mach=(0.5, 0.7), alpha=(-1.0, 3.0)):
    rng = np.random.default_rng(seed)
    return [(float(m), float(a)) for m, a in zip(rng.uniform(*mach, n), rng.uniform(*alpha, n))]


def freestream(mach: float, alpha_deg: float, ncell: int) -> np.ndarray:
    """The reference's free-stream state (gpu_init.cu:79-86), non-dimensional."""
    a = alpha_deg * 3.14159265358979 / 180.0
    rho_e = 1.0 / (GAMMA * (GAMMA - 1.0) * mach * mach) + 0.5
    w = np.empty((ncell, 4))
    w[:, 0] = 1.0
    w[:, 1] = math.cos(a)
    w[:, 2] = math.sin(a)
    w[:, 3] = rho_e
    return w


@dataclass
class SolverSettings:
    """Solver settings shared by every run of the pipeline.

    The reference limiter chatters: its residual stalls between 1e-3 and 1e-2
    on the 256 x 64 O-grid.  The default is the smooth (Venkatakrishnan-type)
    limiter option with K = 10, frozen once Resd reaches 1e-3: over M 0.575 to
    0.70 and alpha -0.1 to 3 every case then falls to 1e-4 in FP32 within 40k
    iterations and on to 1e-6 in FP64.  (K = 5 or 20 without the freeze
    stalls near 1e-3 at M 0.69-0.70, alpha 2.8-3; K = 50 and 200 converge
    where they converge but drift away below M 0.54; nothing here converges at
    M 0.52-0.54 on this mesh, where the residual grows again after ~5k
    iterations.)  ``switch_resd`` > 0 runs FP32 down to that level and FP64
    below it (FP32 states stall near 2e-5); it must stay above the freeze
    level, because frozen limiter values do not carry across precisions.
    ``refreeze_resd`` > 0 stops at that level and continues from the state
    reached in a new solver whose limiter values are frozen after its first
    iteration, i.e. recomputed from a nearly converged state: a run then
    depends less on the state it froze its limiter values on first; that
    second solver runs in ``tail_precision`` (None: ``precision``), which is
    how a run goes below the FP32 floor with frozen limiter values.
    ``irs_eps``, ``positivity_fix`` and ``first_order_iters`` are the solver
    options of the same names."""
    cfl: float = 3.0
    freeze: int = 0
    freeze_resd: float = 1e-3
    precision: int = e2d.E2D_FP32
    limiter: int = 1
    limiter_k: float = 10.0
    switch_resd: float = 0.0
    refreeze_resd: float = 0.0
    tail_precision: int | None = None
    irs_eps: float = 0.8
    positivity_fix: int = 0
    first_order_iters: int = 0

    def params(self, mach, alpha, maxstep=100000, precision=None):
        return e2d.default_params(ma=mach, alpha_deg=alpha, cfl=self.cfl,
                                  precision=self.precision if precision is None else precision,
                                  ordering=e2d.E2D_ORDER_MORTON, limiter_freeze=self.freeze, maxstep=maxstep,
                                  limiter=self.limiter, limiter_k=self.limiter_k,
                                  limiter_freeze_resd=self.freeze_resd, irs_eps=self.irs_eps,
                                  positivity_fix=self.positivity_fix, first_order_iters=self.first_order_iters)


def generate(mesh, conds, settings: SolverSettings, iters: int, chunk: int = 128, log=print):
    """Steady states for every condition (batched solves of `iters` iterations)."""
    states, info = [], []
    for c0 in range(0, len(conds), chunk):
        part = conds[c0:c0 + chunk]
        params = [settings.params(m, a, maxstep=iters) for m, a in part]
        b = e2d.Batch([mesh] * len(part), params)
        t0 = time.perf_counter()
        try:
            b.step(iters)
        except E2DError as exc:  # the other cases ran all their iterations; the diverged ones are left out later
            log(f"generate: {exc}")
        dt = time.perf_counter() - t0
        for c in range(len(part)):
            states.append(b.state(c))
            h = b.history(c)
            info.append({"mach": part[c][0], "alpha": part[c][1], "resd": float(h[-1])})
        log(f"generate: cases {c0}..{c0 + len(part) - 1}: {iters} iterations in {dt:.1f} s, "
            f"Resd median {np.median([i['resd'] for i in info[c0:]]):.2e}")
        b.close()
    return states, info


class Dataset:
    """Normalised features and targets of a set of solutions on one mesh."""

    def __init__(self, mesh, conds, states, fourier_seed: int = 3, sigma: float = 1.0):
        self.fourier_seed, self.sigma = fourier_seed, sigma
        feats = [e2d.MLP.features(mesh, m, a, fourier_seed, sigma) for m, a in conds]
        x = np.concatenate(feats)
        self.x_mean = np.zeros(32, np.float32)
        self.x_std = np.ones(32, np.float32)
        self.x_mean[:6] = x[:, :6].mean(axis=0)
        self.x_std[:6] = np.maximum(x[:, :6].std(axis=0), 1e-6)
        tgt = np.concatenate([s - freestream(m, a, s.shape[0]) for (m, a), s in zip(conds, states)])
        self.t_scale = np.maximum(tgt.std(axis=0), 1e-6)
        self.x = self.normalise(x)
        self.t = (tgt / self.t_scale).astype(np.float32)

    def normalise(self, x):
        return ((x - self.x_mean) / self.x_std).astype(np.float32)

    def to_json(self):
        return {"x_mean": self.x_mean.tolist(), "x_std": self.x_std.tolist(), "t_scale": self.t_scale.tolist(),
                "fourier_seed": self.fourier_seed, "sigma": self.sigma}


def train(ds: Dataset, steps: int, batch: int = 65536, nhidden: int = 5, lr: float = 1e-3, seed: int = 3,
          lr_final: float | None = None, chunk: int = 250, log=print):
    """Adam steps on random batches.  With lr_final, the step size follows a
    cosine from lr down to lr_final, set every `chunk` steps."""
    net = e2d.MLP(nhidden=nhidden, batch=batch, seed=seed, lr=lr)
    net.set_data(ds.x, ds.t)
    t0 = time.perf_counter()
    if lr_final is None:
        loss = net.train(steps)
    else:
        parts = []
        for k0 in range(0, steps, chunk):
            frac = (k0 + 0.5 * min(chunk, steps - k0)) / steps
            net.set_lr(lr_final + 0.5 * (lr - lr_final) * (1.0 + np.cos(np.pi * frac)))
            parts.append(net.train(min(chunk, steps - k0)))
        loss = np.concatenate(parts)
    dt = time.perf_counter() - t0
    log(f"train: {steps} steps of batch {batch} in {dt:.1f} s, loss {loss[:10].mean():.3e} -> {loss[-100:].mean():.3e}")
    return net, loss, dt


def predict(net, ds: Dataset, mesh, mach, alpha):
    x = ds.normalise(e2d.MLP.features(mesh, mach, alpha, ds.fourier_seed, ds.sigma))
    y = net.forward(x).astype(np.float64) * ds.t_scale
    return freestream(mach, alpha, x.shape[0]) + y


def run_to_drop(mesh, mach, alpha, settings: SolverSettings, target, maxit, w0=None, epsm=None):
    s = e2d.Solver(mesh, settings.params(mach, alpha, maxstep=maxit))
    cl0, cd0 = float("nan"), float("nan")
    if w0 is not None:
        s.set_state(w0)
        cl0, cd0 = s.forces()
    if epsm is not None:
        s.set_residual_norm(epsm)
    t0 = time.perf_counter()
    stop = max(target, settings.refreeze_resd)
    h1 = np.zeros(0)  # history of the first solver once the second one runs
    error = None
    tail_wall = 0.0
    try:
        if settings.switch_resd > 0.0:
            h = s.solve_mixed(maxit, stop, settings.switch_resd)
        else:
            h = s.solve(maxit, stop)
        ok = bool(len(h) and h[-1] <= target)
        if stop > target and len(h) and h[-1] <= stop and len(h) < maxit:
            # second freeze: a new solver from the state reached, limiter
            # values frozen after its first iteration
            w, norm = s.state(), s.residual_norm()
            h1 = np.asarray(h, np.float64)
            s.close()
            p2 = settings.params(mach, alpha, maxstep=maxit - len(h), precision=settings.tail_precision)
            p2.limiter_freeze_resd = 1.0
            p2.first_order_iters = 0
            s = e2d.Solver(mesh, p2)
            s.set_state(w)
            s.set_residual_norm(norm)
            t_tail = time.perf_counter()
            h2 = s.solve(maxit - len(h), target)
            tail_wall = time.perf_counter() - t_tail
            h = np.concatenate([h1, h2])
            ok = bool(len(h2) and h2[-1] <= target)
    except E2DError as exc:
        h, ok, error = np.concatenate([h1, s.history()]), False, str(exc)
    wall = time.perf_counter() - t0
    cl, cd = s.forces() if ok else (float("nan"), float("nan"))
    h = np.asarray(h, np.float64)

    def first_below(level):
        k = np.flatnonzero(h <= level)
        return int(k[0]) + 1 if len(k) else None

    out = {"iterations": int(len(h)), "wall_s": wall, "converged": ok, "error": error, "cl": cl, "cd": cd,
           "first_resd": float(h[0]) if len(h) else float("nan"), "epsm": s.residual_norm(),
           "start_cl": cl0, "start_cd": cd0,
           "iterations_to": {f"{lv:.0e}": first_below(lv) for lv in (1e-2, 1e-3, 1e-4, 1e-5)},
           "tail_iterations": int(len(h) - len(h1)) if len(h1) else 0, "tail_wall_s": tail_wall,
           "reached": float(np.min(h)) if len(h) else None,
           "history_every_1000": [float(v) for v in h[999::1000]]}
    s.close()
    return out


def run_budget(mesh, mach, alpha, settings: SolverSettings, budget: int, w0=None, epsm=None, every: int = 5000):
    """A fixed number of iterations (in ``settings.precision``) from the free
    stream or from w0, for cases whose drop is out of reach of the budget:
    the residual history, the iterations at which it first reaches each level,
    and CL / CD every ``every`` iterations."""
    s = e2d.Solver(mesh, settings.params(mach, alpha, maxstep=budget + 10))
    if w0 is not None:
        s.set_state(w0)
    if epsm is not None:
        s.set_residual_norm(epsm)
    forces, error = [], None
    t0 = time.perf_counter()
    try:
        for k0 in range(0, budget, every):
            s.step(min(every, budget - k0))
            cl, cd = s.forces()
            forces.append((k0 + min(every, budget - k0), cl, cd))
    except E2DError as exc:
        error = str(exc)
    wall = time.perf_counter() - t0
    h = s.history()

    def first_below(level):
        k = np.flatnonzero(h <= level)
        return int(k[0]) + 1 if len(k) else None

    out = {"iterations": int(len(h)), "wall_s": wall, "error": error, "epsm": s.residual_norm(),
           "first_resd": float(h[0]) if len(h) else None, "final_resd": float(h[-1]) if len(h) else None,
           "iterations_to": {f"{lv:.0e}": first_below(lv) for lv in (1e-1, 1e-2, 1e-3, 1e-4, 1e-5)},
           "forces": forces, "history_every_1000": [float(v) for v in h[999::1000]]}
    s.close()
    return out


def physical(w, gamma: float = GAMMA) -> bool:
    """Every cell finite with positive density and pressure."""
    w = np.asarray(w, np.float64)
    if not np.all(np.isfinite(w)) or not np.all(w[:, 0] > 0):
        return False
    p = (gamma - 1.0) * (w[:, 3] - 0.5 * (w[:, 1] ** 2 + w[:, 2] ** 2) / w[:, 0])
    return bool(np.all(p > 0))


def run_warm(mesh, mach, alpha, settings: SolverSettings, target, maxit, w_pred, epsm=None):
    """The plain solver from a predicted state, with the free stream as the
    fallback: a prediction that is not physical in every cell is not used, and
    a warm run that stops with an error (diverged) is run again from the free
    stream, its iterations and time counted with the fallback's (in
    ``iterations``, ``wall_s`` and every ``iterations_to`` entry; the attempt
    alone in ``failed_attempt``).  ``fallback`` in the result says which, or
    is None."""
    if not physical(w_pred):
        out = run_to_drop(mesh, mach, alpha, settings, target, maxit, epsm=epsm)
        out["fallback"] = "prediction not physical"
        return out
    warm = run_to_drop(mesh, mach, alpha, settings, target, maxit, w0=w_pred, epsm=epsm)
    if warm["error"] is None:
        warm["fallback"] = None
        return warm
    free = run_to_drop(mesh, mach, alpha, settings, target, maxit, epsm=epsm)
    # every count of the result includes the failed attempt's cost; the
    # attempt's own figures are kept beside them
    free["failed_attempt"] = {"iterations": warm["iterations"], "wall_s": warm["wall_s"]}
    free["iterations"] += warm["iterations"]
    free["wall_s"] += warm["wall_s"]
    free["iterations_to"] = {k: (v + warm["iterations"] if v is not None else None)
                             for k, v in free["iterations_to"].items()}
    free["start_cl"], free["start_cd"] = warm["start_cl"], warm["start_cd"]
    free["fallback"] = f"warm run failed: {warm['error']}"
    return free


def evaluate(net, ds, mesh, conds, settings: SolverSettings, target: float, maxit: int, log=print):
    rows = []
    for m, a in conds:
        free = run_to_drop(mesh, m, a, settings, target, maxit)
        warm_state = predict(net, ds, mesh, m, a)
        warm = run_warm(mesh, m, a, settings, target, maxit, warm_state, epsm=free["epsm"])
        r = {"mach": m, "alpha": a, "free": free, "warm": warm,
             "speedup_wall": free["wall_s"] / warm["wall_s"] if warm["converged"] else float("nan"),
             "speedup_iter": free["iterations"] / max(1, warm["iterations"]) if warm["converged"] else float("nan"),
             "dcl": abs(warm["cl"] - free["cl"]), "dcd": abs(warm["cd"] - free["cd"])}
        rows.append(r)
        log(f"eval M{m:.3f} a{a:+.2f}: free {free['iterations']} its {free['wall_s']:.2f} s | warm "
            f"{warm['iterations']} its {warm['wall_s']:.2f} s (first Resd {warm['first_resd']:.2e}) | "
            f"x{r['speedup_wall']:.2f} wall, dCL {r['dcl']:.1e} dCD {r['dcd']:.1e} | predicted CL error "
            f"{abs(warm['start_cl'] - free['cl']):.1e} | its to 1e-3/1e-4/1e-5 free "
            f"{'/'.join(str(v) for v in list(free['iterations_to'].values())[1:])} warm "
            f"{'/'.join(str(v) for v in list(warm['iterations_to'].values())[1:])}"
            + (f" | fallback: {warm['fallback']}" if warm["fallback"] else ""))
    return rows


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--ni", type=int, default=256)
    ap.add_argument("--nj", type=int, default=64)
    ap.add_argument("--ntrain", type=int, default=256)
    ap.add_argument("--nheld", type=int, default=32)
    ap.add_argument("--neval", type=int, default=8, help="held-out conditions timed one by one")
    ap.add_argument("--gen-iters", type=int, default=80000)
    ap.add_argument("--steps", type=int, default=60000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--nhidden", type=int, default=8, help="hidden layers of width 256")
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--lr-final", type=float, default=1e-5,
                    help="cosine decay of the Adam step size down to this value (<= 0: constant)")
    ap.add_argument("--target", type=float, default=1e-6)
    ap.add_argument("--maxit", type=int, default=120000)
    ap.add_argument("--mach", type=float, nargs=2, default=(0.575, 0.70))
    ap.add_argument("--alpha", type=float, nargs=2, default=(-1.0, 3.0))
    ap.add_argument("--eval", choices=["fp64", "switch", "tail"], default="fp64",
                    help="timed runs in FP64; FP32 down to 2e-3 and FP64 below; or FP32 down to the "
                         "--refreeze level and a new FP64 solver (limiter values frozen again) below")
    ap.add_argument("--limiter", type=int, default=1, help="limiter option of every solve (1: per-face "
                    "Venkatakrishnan, 3: cell-wise Venkatakrishnan)")
    ap.add_argument("--limiter-k", type=float, default=10.0)
    ap.add_argument("--cfl", type=float, default=3.0)
    ap.add_argument("--irs-eps", type=float, default=0.8)
    ap.add_argument("--freeze", type=float, default=1e-3, help="limiter values frozen at this Resd")
    ap.add_argument("--freeze-after", type=int, default=0,
                    help="... or at this iteration, whichever comes first (0: level only)")
    ap.add_argument("--refreeze", type=float, default=1e-5,
                    help="freeze the limiter values again, from the state at this level (0: off)")
    ap.add_argument("--eval-mesh", type=int, nargs=2, default=None, metavar=("NI", "NJ"),
                    help="also predict on this finer O-grid and compare free and warm runs there")
    ap.add_argument("--eval-cond", type=float, nargs=2, default=(0.78, 2.0), metavar=("MACH", "ALPHA"))
    ap.add_argument("--budget", type=int, default=100000, help="FP32 iterations of each run on --eval-mesh")
    ap.add_argument("--eval-freeze", type=float, default=None,
                    help="limiter freeze level of the --eval-mesh runs (default --freeze; 0: never)")
    ap.add_argument("--cache", default=None,
                    help="npz file of the generated training / held-out states: loaded when it exists and "
                         "matches the mesh and conditions, else written after generation")
    ap.add_argument("--json", default=None)
    args = ap.parse_args(argv)
    log = lambda s: print(s, file=sys.stderr, flush=True)  # noqa: E731
    mesh = e2d.Mesh.ogrid(args.ni, args.nj, seed=1)
    train_c = conditions(args.ntrain, 3, tuple(args.mach), tuple(args.alpha))
    held_c = conditions(args.nheld, 4, tuple(args.mach), tuple(args.alpha))
    scheme = dict(cfl=args.cfl, limiter=args.limiter, limiter_k=args.limiter_k, irs_eps=args.irs_eps,
                  freeze_resd=args.freeze, freeze=args.freeze_after)
    gen = SolverSettings(precision=e2d.E2D_FP32, **scheme)
    key = np.array([args.ni, args.nj, args.gen_iters] + [v for c in train_c + held_c for v in c], np.float64)
    cached = None
    if args.cache:
        try:
            z = np.load(args.cache)
            if z["key"].shape == key.shape and np.array_equal(z["key"], key):
                cached = z
        except (OSError, KeyError, ValueError):
            cached = None
    if cached is not None:
        states = list(cached["train"])
        info = []
        log(f"generate: {len(states)} training states from {args.cache}")
    else:
        states, info = generate(mesh, train_c, gen, args.gen_iters, log=log)
    # a generated state that is not physical (a case that diverged) is not
    # a training target
    all_states = states
    keep = [k for k, w in enumerate(states) if physical(w)]
    if len(keep) < len(states):
        log(f"generate: {len(states) - len(keep)} of {len(states)} training cases diverged and are left out")
    train_c, states = [train_c[k] for k in keep], [states[k] for k in keep]
    ds = Dataset(mesh, train_c, states)
    net, loss, t_train = train(ds, args.steps, args.batch, nhidden=args.nhidden, lr=args.lr,
                               lr_final=args.lr_final if args.lr_final > 0 else None, log=log)
    # prediction error on the held-out conditions against their FP32 solutions
    if cached is not None:
        held_states = list(cached["held"])
    else:
        held_states, _ = generate(mesh, held_c, gen, args.gen_iters, log=log)
        if args.cache:
            np.savez(args.cache, key=key, train=np.array(all_states), held=np.array(held_states))
    errs = []
    for (m, a), w in zip(held_c, held_states):
        if not physical(w):
            continue
        p = predict(net, ds, mesh, m, a)
        errs.append(float(np.sqrt(np.mean((p - w) ** 2, axis=0)).max() / np.abs(w).max()))
    log(f"held-out prediction RMS error (max over components, rel. to max |W|): median {np.median(errs):.2e}")
    if args.eval == "tail":
        ev = SolverSettings(precision=e2d.E2D_FP32, tail_precision=e2d.E2D_FP64, refreeze_resd=args.refreeze,
                            **scheme)
    else:
        ev = SolverSettings(precision=e2d.E2D_FP64, switch_resd=2e-3 if args.eval == "switch" else 0.0,
                            refreeze_resd=args.refreeze, **scheme)
    rows = evaluate(net, ds, mesh, held_c[:args.neval], ev, args.target, args.maxit, log=log) if args.neval else []
    conv = [r for r in rows if r["warm"]["converged"] and r["free"]["converged"]]
    large = None
    if args.eval_mesh:
        # the network trained on the coarse mesh evaluated at the centroids of
        # a finer one; both runs take the same FP32 budget there
        big = e2d.Mesh.ogrid(args.eval_mesh[0], args.eval_mesh[1], seed=1)
        m, a = args.eval_cond
        t0 = time.perf_counter()
        w_pred = predict(net, ds, big, m, a)
        t_pred = time.perf_counter() - t0
        fine_scheme = dict(scheme)
        if args.eval_freeze is not None:
            fine_scheme.update(freeze_resd=args.eval_freeze, freeze=0)
        fine = SolverSettings(precision=e2d.E2D_FP32, **fine_scheme)
        free = run_budget(big, m, a, fine, args.budget)
        warm = run_budget(big, m, a, fine, args.budget, w0=w_pred if physical(w_pred) else None, epsm=free["epsm"])
        large = {"mesh": f"{args.eval_mesh[0]}x{args.eval_mesh[1]}", "mach": m, "alpha": a, "budget": args.budget,
                 "predict_seconds": t_pred, "prediction_physical": physical(w_pred), "free": free, "warm": warm}
        log(f"large mesh {large['mesh']} M{m} a{a}: free {free['iterations_to']} final {free['final_resd']:.2e} | "
            f"warm {warm['iterations_to']} final {warm['final_resd']:.2e} (first {warm['first_resd']:.2e})")
    summary = {
        "mesh": f"{args.ni}x{args.nj}", "ntrain": args.ntrain, "nheld": args.nheld, "mach": list(args.mach),
        "alpha": list(args.alpha), "gen_iters": args.gen_iters, "train_steps": args.steps, "batch": args.batch, "nhidden": args.nhidden,
        "lr": args.lr, "lr_final": args.lr_final,
        "train_seconds": t_train, "final_loss": float(loss[-100:].mean()),
        "heldout_pred_err_median": float(np.median(errs)), "target_drop": args.target,
        "eval_precision": args.eval, "refreeze": args.refreeze, "scheme": scheme,
        "evaluated": len(rows), "both_converged": len(conv),
        "fallbacks": sum(1 for r in rows if r["warm"]["fallback"]),
        "speedup_wall_median": float(np.median([r["speedup_wall"] for r in conv])) if conv else None,
        "speedup_iter_median": float(np.median([r["speedup_iter"] for r in conv])) if conv else None,
        "max_dcl": float(max(r["dcl"] for r in conv)) if conv else None,
        "max_dcd": float(max(r["dcd"] for r in conv)) if conv else None,
        "rows": rows, "large_mesh": large,
    }
    text = json.dumps(summary)
    print(text, flush=True)
    if args.json:
        with open(args.json, "w") as f:
            f.write(text + "\n")
    return summary


if __name__ == "__main__":
    main()

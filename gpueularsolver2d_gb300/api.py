"""Python view of the C ABI: ``Mesh`` and ``Solver`` handles over libeuler2d.

The calls map one to one onto include/euler2d.h; numpy arrays cross the
boundary as plain pointers.  Cell arrays are in file order.
"""
from __future__ import annotations

import ctypes

import numpy as np

from ._lib import (E2D_FP32, E2D_FP64, E2D_LIMITER_CELL_BARTH, E2D_LIMITER_CELL_VENKAT,  # noqa: F401
                   E2D_LIMITER_REFERENCE, E2D_LIMITER_VENKAT, E2D_ORDER_FILE, E2D_ORDER_MORTON, E2D_ORDER_RCM, MeshInfo, Params,
                   check, load)

__all__ = ["Mesh", "Solver", "Batch", "MLP", "Params", "default_params", "read_input", "E2D_FP32", "E2D_FP64",
           "E2D_ORDER_FILE", "E2D_ORDER_MORTON", "E2D_ORDER_RCM"]


def _dp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int32))


def default_params(**kw) -> Params:
    """Reference defaults, with any field overridden by keyword."""
    p = Params()
    check(load().e2d_params_default(ctypes.byref(p)))
    names = {f[0] for f in Params._fields_}
    for k, v in kw.items():
        if k not in names:
            raise TypeError(f"unknown solver parameter {k!r}")
        if k == "rk_coef":
            for i, c in enumerate(v):
                p.rk_coef[i] = c
        else:
            setattr(p, k, v)
    return p


def state_integrals(mesh: "Mesh", params: Params, w) -> dict:
    """FP64 integrals (cl, cd, mass, mass_flux_far, mass_flux_wall) of a state
    [ncell, 4] in the mesh's cell order, computed on the host (no GPU)."""
    from ._lib import Integrals
    w = np.ascontiguousarray(w, np.float64)
    if w.size != 4 * mesh.info(params.wall_box).ncell:
        raise ValueError("need a [ncell, 4] state")
    out = Integrals()
    check(load().e2d_state_integrals(mesh._h, ctypes.byref(params), _dp(w), ctypes.byref(out)))
    return out.as_dict()


def read_input(path: str, p: Params | None = None) -> Params:
    p = p or default_params()
    check(load().e2d_input_read(path.encode(), ctypes.byref(p)))
    return p


class Mesh:
    def __init__(self, handle: int):
        self._h = ctypes.c_void_p(handle)

    @classmethod
    def read(cls, path: str) -> "Mesh":
        h = ctypes.c_void_p()
        check(load().e2d_mesh_read(path.encode(), ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def from_arrays(cls, x, y, tri) -> "Mesh":
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        tri = np.ascontiguousarray(tri, np.int32).reshape(-1)
        h = ctypes.c_void_p()
        check(load().e2d_mesh_from_arrays(len(x), len(tri) // 3, _dp(x), _dp(y), _ip(tri),
                                          ctypes.byref(h)))
        return cls(h.value)

    @classmethod
    def ogrid(cls, ni: int, nj: int, r_far: float = 20.0, dy_wall: float = 2e-3,
              jitter: float = 0.05, seed: int = 1) -> "Mesh":
        h = ctypes.c_void_p()
        check(load().e2d_mesh_ogrid_naca0012(ni, nj, r_far, dy_wall, jitter, seed, ctypes.byref(h)))
        return cls(h.value)

    def write(self, path: str, binary: bool = False) -> None:
        """Reference .dat text, or the binary cache that Mesh.read also accepts."""
        fn = load().e2d_mesh_write_binary if binary else load().e2d_mesh_write
        check(fn(path.encode(), self._h))

    def info(self, wall_box: float = 2.0) -> MeshInfo:
        i = MeshInfo()
        check(load().e2d_mesh_info_get(self._h, wall_box, ctypes.byref(i)))
        return i

    def topology(self, wall_box: float = 2.0):
        """(edge_int[nedge,7], edge_dbl[nedge,5], cell_int[ncell,7], cell_dbl[ncell,3])."""
        inf = self.info(wall_box)
        ei = np.zeros((inf.nedge, 7), np.int32)
        ed = np.zeros((inf.nedge, 5))
        ci = np.zeros((inf.ncell, 7), np.int32)
        cd = np.zeros((inf.ncell, 3))
        check(load().e2d_mesh_topology(self._h, wall_box, _ip(ei), _dp(ed), _ip(ci), _dp(cd)))
        return ei, ed, ci, cd

    def nodes(self):
        inf = self.info()
        x = np.zeros(inf.nnode)
        y = np.zeros(inf.nnode)
        tri = np.zeros((inf.ncell, 3), np.int32)
        check(load().e2d_mesh_nodes(self._h, _dp(x), _dp(y), _ip(tri)))
        return x, y, tri

    def order(self, ordering: int) -> np.ndarray:
        perm = np.zeros(self.info().ncell, np.int32)
        check(load().e2d_mesh_order(self._h, ordering, _ip(perm)))
        return perm

    def close(self) -> None:
        if self._h:
            load().e2d_mesh_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    def __init__(self, mesh: Mesh, params: Params):
        self.mesh = mesh
        self.params = params
        self.ncell = mesh.info(params.wall_box).ncell
        h = ctypes.c_void_p()
        check(load().e2d_solver_create(mesh._h, ctypes.byref(params), ctypes.byref(h)))
        self._h = h

    def step(self, n: int) -> None:
        check(load().e2d_step(self._h, n))

    def solve(self, max_steps: int, epsl: float) -> np.ndarray:
        hist = np.zeros(max(1, max_steps))
        n = ctypes.c_int32()
        check(load().e2d_solve(self._h, max_steps, epsl, _dp(hist), ctypes.byref(n)))
        return hist[: n.value].copy()

    def set_precision(self, precision: int) -> None:
        """Switch the stencil precision in place (state, step count, residual
        normalisation and history carry over)."""
        check(load().e2d_set_precision(self._h, precision))

    def solve_mixed(self, max_steps: int, epsl: float, switch: float = 1e-4) -> np.ndarray:
        """FP32 iterations until Resd <= switch, then FP64 until Resd <= epsl:
        most of the work at FP32 speed, the end below the FP32 rounding floor.
        Returns the residuals of both phases."""
        self.set_precision(E2D_FP32)
        h1 = self.solve(max_steps, max(switch, epsl))
        rest = max_steps - len(h1)
        if rest <= 0 or (len(h1) and h1[-1] <= epsl):
            return h1
        self.set_precision(E2D_FP64)
        return np.concatenate([h1, self.solve(rest, epsl)])

    def progress(self):
        st = ctypes.c_int32()
        r = ctypes.c_double()
        check(load().e2d_progress(self._h, ctypes.byref(st), ctypes.byref(r)))
        return st.value, r.value

    def history(self) -> np.ndarray:
        n = ctypes.c_int32()
        check(load().e2d_residual_history(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(max(1, n.value))
        check(load().e2d_residual_history(self._h, _dp(out), n.value, ctypes.byref(n)))
        return out[: n.value]

    def set_residual_norm(self, epsm: float) -> None:
        check(load().e2d_set_residual_norm(self._h, epsm))

    def residual_norm(self) -> float:
        v = ctypes.c_double()
        check(load().e2d_get_residual_norm(self._h, ctypes.byref(v)))
        return v.value

    def state(self) -> np.ndarray:
        w = np.zeros((self.ncell, 4))
        check(load().e2d_get_state(self._h, _dp(w)))
        return w

    def state_into(self, out: np.ndarray) -> None:
        """Copy the state into a caller buffer (e.g. pinned memory), [ncell, 4] float64."""
        if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != 4 * self.ncell:
            raise ValueError("need a C-contiguous float64 [ncell, 4] buffer")
        check(load().e2d_get_state(self._h, _dp(out)))

    def set_state(self, w) -> None:
        w = np.ascontiguousarray(w, np.float64).reshape(self.ncell, 4)
        check(load().e2d_set_state(self._h, _dp(w)))

    def forces(self):
        cl = ctypes.c_double()
        cd = ctypes.c_double()
        check(load().e2d_forces(self._h, ctypes.byref(cl), ctypes.byref(cd)))
        return cl.value, cd.value

    def integrals(self) -> dict:
        """FP64 integrals of the current state: cl, cd, mass, mass_flux_far,
        mass_flux_wall (e2d_integrals)."""
        from ._lib import Integrals
        out = Integrals()
        check(load().e2d_solver_integrals(self._h, ctypes.byref(out)))
        return out.as_dict()

    def write_residual_plt(self, path: str) -> None:
        check(load().e2d_write_residual_plt(self._h, path.encode()))

    def last_device_ms(self) -> float:
        v = ctypes.c_double()
        check(load().e2d_last_device_ms(self._h, ctypes.byref(v)))
        return v.value

    def launches_per_iteration(self) -> int:
        v = ctypes.c_int32()
        check(load().e2d_launches_per_iteration(self._h, ctypes.byref(v)))
        return v.value

    def profile_passes(self, iters: int):
        """Per-pass device ms summed over iters iterations, and launch counts."""
        ms = np.zeros(5)
        nl = np.zeros(5, np.int32)
        check(load().e2d_profile_passes(self._h, iters, _dp(ms), _ip(nl)))
        return ms, nl

    def close(self) -> None:
        if self._h:
            load().e2d_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Many independent cases advanced together (e2d_batch_* in include/euler2d.h)."""

    def __init__(self, meshes, params):
        self.meshes = list(meshes)
        self.params = list(params)
        n = len(self.meshes)
        handles = (ctypes.c_void_p * n)(*[m._h.value for m in self.meshes])
        parr = (Params * n)(*self.params)
        h = ctypes.c_void_p()
        check(load().e2d_batch_create(handles, parr, n, ctypes.byref(h)))
        self._h = h
        self.ncells = [m.info(p.wall_box).ncell for m, p in zip(self.meshes, self.params)]

    @classmethod
    def tuned(cls, meshes, params, cache_path: str | None = None, iters: int = 16):
        """Batch with the cell order and launch shape picked by the autotuner
        (e2d_batch_create_tuned); .ordering holds the order chosen."""
        self = cls.__new__(cls)
        self.meshes = list(meshes)
        self.params = list(params)
        n = len(self.meshes)
        handles = (ctypes.c_void_p * n)(*[m._h.value for m in self.meshes])
        parr = (Params * n)(*self.params)
        h = ctypes.c_void_p()
        order = ctypes.c_int32()
        check(load().e2d_batch_create_tuned(handles, parr, n, cache_path.encode() if cache_path else None, iters,
                                            ctypes.byref(h), ctypes.byref(order)))
        self._h = h
        self.ordering = order.value
        self.ncells = [m.info(p.wall_box).ncell for m, p in zip(self.meshes, self.params)]
        return self

    def step(self, n: int) -> None:
        check(load().e2d_batch_step(self._h, n))

    def solve(self, max_steps: int, epsl: float) -> np.ndarray:
        out = np.zeros(len(self.meshes), np.int32)
        check(load().e2d_batch_solve(self._h, max_steps, epsl, _ip(out)))
        return out

    def info(self):
        nc = ctypes.c_int32()
        nt = ctypes.c_int64()
        npad = ctypes.c_int64()
        check(load().e2d_batch_info(self._h, ctypes.byref(nc), ctypes.byref(nt), ctypes.byref(npad)))
        return nc.value, nt.value, npad.value

    def state(self, c: int) -> np.ndarray:
        w = np.zeros((self.ncells[c], 4))
        check(load().e2d_batch_get_state(self._h, c, _dp(w)))
        return w

    def set_state(self, c: int, w) -> None:
        w = np.ascontiguousarray(w, np.float64).reshape(self.ncells[c], 4)
        check(load().e2d_batch_set_state(self._h, c, _dp(w)))

    def progress(self, c: int):
        st = ctypes.c_int32()
        r = ctypes.c_double()
        hl = ctypes.c_int32()
        check(load().e2d_batch_progress(self._h, c, ctypes.byref(st), ctypes.byref(r), ctypes.byref(hl)))
        return st.value, r.value, hl.value

    def history(self, c: int) -> np.ndarray:
        n = ctypes.c_int32()
        check(load().e2d_batch_residual_history(self._h, c, None, 0, ctypes.byref(n)))
        out = np.zeros(max(1, n.value))
        check(load().e2d_batch_residual_history(self._h, c, _dp(out), n.value, ctypes.byref(n)))
        return out[: n.value]

    def forces(self, c: int):
        cl = ctypes.c_double()
        cd = ctypes.c_double()
        check(load().e2d_batch_forces(self._h, c, ctypes.byref(cl), ctypes.byref(cd)))
        return cl.value, cd.value

    def set_launch(self, block: int, grid: int = 0) -> None:
        check(load().e2d_batch_set_launch(self._h, block, grid))

    def launch(self):
        b = ctypes.c_int32()
        g = ctypes.c_int32()
        check(load().e2d_batch_get_launch(self._h, ctypes.byref(b), ctypes.byref(g)))
        return b.value, g.value

    def autotune(self, cache_path: str | None = None, iters: int = 16):
        b = ctypes.c_int32()
        g = ctypes.c_int32()
        ms = ctypes.c_double()
        check(load().e2d_batch_autotune(self._h, cache_path.encode() if cache_path else None, iters,
                                        ctypes.byref(b), ctypes.byref(g), ctypes.byref(ms)))
        return b.value, g.value, ms.value

    def last_device_ms(self) -> float:
        v = ctypes.c_double()
        check(load().e2d_batch_last_device_ms(self._h, ctypes.byref(v)))
        return v.value

    def launches_per_iteration(self) -> int:
        v = ctypes.c_int32()
        check(load().e2d_batch_launches_per_iteration(self._h, ctypes.byref(v)))
        return v.value

    def close(self) -> None:
        if self._h:
            load().e2d_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _fp(a: np.ndarray):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class MLP:
    """The warm-start coordinate MLP (e2d_mlp_* in include/euler2d.h)."""

    INPUTS = 32
    FEATURES = 22

    def __init__(self, nhidden: int = 5, batch: int = 65536, seed: int = 3, lr: float = 1e-3):
        from ._lib import MLPConfig
        c = MLPConfig()
        check(load().e2d_mlp_config_default(ctypes.byref(c)))
        c.nhidden, c.batch, c.seed, c.lr = nhidden, batch, seed, lr
        self.config = c
        h = ctypes.c_void_p()
        check(load().e2d_mlp_create(ctypes.byref(c), ctypes.byref(h)))
        self._h = h

    def param_count(self) -> int:
        n = ctypes.c_int64()
        check(load().e2d_mlp_param_count(self._h, ctypes.byref(n)))
        return n.value

    def params(self) -> np.ndarray:
        p = np.zeros(self.param_count(), np.float32)
        check(load().e2d_mlp_get_params(self._h, _fp(p)))
        return p

    def set_params(self, p) -> None:
        p = np.ascontiguousarray(p, np.float32)
        check(load().e2d_mlp_set_params(self._h, _fp(p)))

    def set_data(self, x, t) -> None:
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.INPUTS)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, 4)
        check(load().e2d_mlp_set_data(self._h, x.shape[0], _fp(x), _fp(t)))

    def set_lr(self, lr: float) -> None:
        """Adam step size of the following training steps."""
        check(load().e2d_mlp_set_lr(self._h, lr))

    def train(self, steps: int, record_loss: bool = True) -> np.ndarray:
        loss = np.zeros(steps)
        check(load().e2d_mlp_train(self._h, steps, _dp(loss) if record_loss else None))
        return loss

    def forward(self, x) -> np.ndarray:
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.INPUTS)
        y = np.zeros((x.shape[0], 4), np.float32)
        check(load().e2d_mlp_forward(self._h, x.shape[0], _fp(x), _fp(y)))
        return y

    def gradient(self, x, t):
        x = np.ascontiguousarray(x, np.float32).reshape(-1, self.INPUTS)
        t = np.ascontiguousarray(t, np.float32).reshape(-1, 4)
        g = np.zeros(self.param_count(), np.float32)
        loss = ctypes.c_double()
        check(load().e2d_mlp_gradient(self._h, _fp(x), _fp(t), ctypes.byref(loss), _fp(g)))
        return loss.value, g

    @staticmethod
    def features(mesh: "Mesh", mach: float, alpha_deg: float, seed: int = 3, sigma: float = 1.0,
                 wall_box: float = 2.0) -> np.ndarray:
        n = mesh.info(wall_box).ncell
        out = np.zeros((n, MLP.INPUTS), np.float32)
        check(load().e2d_mlp_features(mesh._h, wall_box, mach, alpha_deg, seed, sigma, _fp(out)))
        return out

    def close(self) -> None:
        if self._h:
            load().e2d_mlp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

"""ctypes view of the CPU oracle (liboracle.so) and of the reference harness.

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline leg of bench.py, never by the product package.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


class OrParams(ctypes.Structure):
    """Mirror of ``or_params`` in e2d_oracle.h."""
    _fields_ = [
        ("ma", ctypes.c_double), ("alpha_deg", ctypes.c_double), ("gamma", ctypes.c_double),
        ("pin", ctypes.c_double), ("tin", ctypes.c_double), ("cfl", ctypes.c_double),
        ("epsl", ctypes.c_double), ("maxstep", ctypes.c_int), ("rk_stages", ctypes.c_int),
        ("rk_coef", ctypes.c_double * 8), ("irs_eps", ctypes.c_double),
        ("irs_sweeps", ctypes.c_int), ("dt_cap", ctypes.c_double),
        ("entropy_eps", ctypes.c_double), ("wall_box", ctypes.c_double),
        ("limiter_freeze", ctypes.c_int), ("limiter", ctypes.c_int), ("limiter_k", ctypes.c_double),
        ("limiter_freeze_resd", ctypes.c_double), ("global_dt", ctypes.c_int),
        ("far_field_fix", ctypes.c_int), ("first_order_iters", ctypes.c_int),
        ("positivity_fix", ctypes.c_int),
    ]


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        import importlib.util
        spec = importlib.util.spec_from_file_location("oracle_build", os.path.join(HERE, "build.py"))
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
        path = mod.build()
        L = ctypes.CDLL(path)
        vp, dp, ip = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int)
        L.or_create.restype = vp
        L.or_create.argtypes = [ctypes.c_int, ctypes.c_int, dp, dp, ip, ctypes.POINTER(OrParams)]
        L.or_create_from_file.restype = vp
        L.or_create_from_file.argtypes = [ctypes.c_char_p, ctypes.POINTER(OrParams)]
        L.or_last_error.restype = ctypes.c_char_p
        for name, args in {
            "or_destroy": [vp], "or_counts": [vp, ip], "or_topology": [vp, ip, dp, ip, dp],
            "or_get_state": [vp, dp], "or_set_state": [vp, dp], "or_get_pta": [vp, dp],
            "or_run": [vp, ctypes.c_int, dp], "or_stage_probe": [vp, dp, dp, dp, dp, dp, dp, dp],
            "or_morton_perm": [vp, ip], "or_rcm_perm": [vp, ip], "or_set_threads": [ctypes.c_int],
            "or_params_default": [ctypes.POINTER(OrParams)],
            "or_roe_flux": [dp, dp, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double, dp],
            "or_far_ghost": [dp, ctypes.c_double, ctypes.c_double, vp, dp],
        }.items():
            getattr(L, name).argtypes = args
        L.or_ogrid_naca0012.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                        ctypes.c_double, ctypes.c_uint64, dp, dp, ip]
        L.or_pis.restype = ctypes.c_double
        L.or_pis.argtypes = [vp]
        L.or_step_count.argtypes = [vp]
        L.or_threads.restype = ctypes.c_int
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _ip(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_int))


def params(**kw) -> OrParams:
    p = OrParams()
    lib().or_params_default(ctypes.byref(p))
    for k, v in kw.items():
        if k == "rk_coef":
            for i, c in enumerate(v):
                p.rk_coef[i] = c
        else:
            setattr(p, k, v)
    return p


def params_from_e2d(ep) -> OrParams:
    """Same settings as an e2d ``Params`` structure."""
    names = [f[0] for f in OrParams._fields_]
    return params(**{n: (list(getattr(ep, n)) if n == "rk_coef" else getattr(ep, n)) for n in names})


class Case:
    def __init__(self, x, y, tri, p: OrParams):
        x = np.ascontiguousarray(x, np.float64)
        y = np.ascontiguousarray(y, np.float64)
        tri = np.ascontiguousarray(tri, np.int32).reshape(-1)
        self.p = p
        self._h = lib().or_create(len(x), len(tri) // 3, _dp(x), _dp(y), _ip(tri), ctypes.byref(p))
        if not self._h:
            raise ValueError(lib().or_last_error().decode())
        c = (ctypes.c_int * 5)()
        lib().or_counts(self._h, c)
        self.ncell, self.nnode, self.nedge, self.nwall, self.nfar = list(c)

    @classmethod
    def from_file(cls, path: str, p: OrParams) -> "Case":
        self = cls.__new__(cls)
        self.p = p
        self._h = lib().or_create_from_file(path.encode(), ctypes.byref(p))
        if not self._h:
            raise ValueError(lib().or_last_error().decode())
        c = (ctypes.c_int * 5)()
        lib().or_counts(self._h, c)
        self.ncell, self.nnode, self.nedge, self.nwall, self.nfar = list(c)
        return self

    def topology(self):
        ei = np.zeros((self.nedge, 7), np.int32)
        ed = np.zeros((self.nedge, 5))
        ci = np.zeros((self.ncell, 7), np.int32)
        cd = np.zeros((self.ncell, 3))
        lib().or_topology(self._h, _ip(ei), _dp(ed), _ip(ci), _dp(cd))
        return ei, ed, ci, cd

    def state(self) -> np.ndarray:
        w = np.zeros((self.ncell, 4))
        lib().or_get_state(self._h, _dp(w))
        return w

    def set_state(self, w) -> None:
        w = np.ascontiguousarray(w, np.float64)
        lib().or_set_state(self._h, _dp(w))

    def run(self, n: int) -> np.ndarray:
        r = np.zeros(max(1, n))
        k = lib().or_run(self._h, n, _dp(r))
        return r[:k].copy()

    def pis(self) -> float:
        return lib().or_pis(self._h)

    def stage_probe(self):
        gh = np.zeros((self.nedge, 4))
        gr = np.zeros((self.ncell, 8))
        um = np.zeros((self.ncell, 8))
        fl = np.zeros((self.nedge, 4))
        sr = np.zeros(self.nedge)
        res = np.zeros((self.ncell, 4))
        dt = np.zeros(self.ncell)
        lib().or_stage_probe(self._h, _dp(gh), _dp(gr), _dp(um), _dp(fl), _dp(sr), _dp(res), _dp(dt))
        return dict(ghost=gh, grad=gr, umm=um, flux=fl, sr=sr, res=res, dt=dt)

    def rcm(self) -> np.ndarray:
        perm = np.zeros(self.ncell, np.int32)
        lib().or_rcm_perm(self._h, _ip(perm))
        return perm

    def far_ghost(self, dw, vectorx: float, vectory: float) -> np.ndarray:
        """Far-field ghost of interior state dw across a face (vectorx, vectory)."""
        dw = np.ascontiguousarray(dw, np.float64)
        out = np.zeros(4)
        lib().or_far_ghost(_dp(dw), vectorx, vectory, self._h, _dp(out))
        return out

    def morton(self) -> np.ndarray:
        perm = np.zeros(self.ncell, np.int32)
        lib().or_morton_perm(self._h, _ip(perm))
        return perm

    def __del__(self):
        try:
            if self._h:
                lib().or_destroy(self._h)
                self._h = None
        except Exception:
            pass


def ogrid(ni: int, nj: int, r_far: float = 20.0, dy_wall: float = 2e-3, jitter: float = 0.05,
          seed: int = 1):
    """The NACA 0012 O-grid (x, y, tri with 1-based node ids), the same mesh as
    the library's generator with the same arguments, made without it."""
    x = np.zeros(ni * (nj + 1))
    y = np.zeros(ni * (nj + 1))
    tri = np.zeros((2 * ni * nj, 3), np.int32)
    if lib().or_ogrid_naca0012(ni, nj, r_far, dy_wall, jitter, seed, _dp(x), _dp(y), _ip(tri)) != 0:
        raise ValueError(lib().or_last_error().decode())
    return x, y, tri


def set_threads(n: int) -> None:
    lib().or_set_threads(n)


def threads() -> int:
    return lib().or_threads()


# ---- reference harness (oracle/_ref/ref_harness) -------------------------

def ref_harness_path() -> str | None:
    """Path of the built reference harness, building it when sources exist."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("build_ref", os.path.join(HERE, "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    try:
        return mod.build()
    except Exception:
        return None


def run_reference(mode: str, mesh_path: str, input_line: str, w_in: np.ndarray | None = None,
                  workdir: str | None = None, trace: bool = False, dump_at=()) -> dict:
    """Run the reference harness in a scratch directory and read its dumps.

    In "gpu" mode, ``trace`` adds ``drou`` (sum of (rho_n - rho_{n-1})^2 of
    every iteration, from the program's own states) and ``dump_at`` adds
    ``w_at`` = {k: state after k iterations}."""
    exe = ref_harness_path()
    if exe is None:
        raise FileNotFoundError("reference sources not available")
    own = workdir is None
    d = workdir or tempfile.mkdtemp(prefix="e2dref_")
    try:
        shutil.copyfile(mesh_path, os.path.join(d, "2822-3k.dat"))
        with open(os.path.join(d, "input.dat"), "w") as f:
            f.write(input_line + "\n")
        if w_in is not None:
            np.ascontiguousarray(w_in, np.float64).tofile(os.path.join(d, "w_in.bin"))
        env = dict(os.environ)
        env.pop("E2D_REF_TRACE", None)
        env.pop("E2D_REF_DUMP_AT", None)
        if trace:
            env["E2D_REF_TRACE"] = "1"
        if dump_at:
            env["E2D_REF_DUMP_AT"] = ",".join(str(int(k)) for k in dump_at)
        res = subprocess.run([exe, mode, d], capture_output=True, text=True, env=env)
        if res.returncode != 0:
            raise RuntimeError(f"reference harness failed: {res.stderr[-2000:]}")
        out = {"stdout": res.stdout}
        for name, dt in [("counts", np.int32), ("edge_i", np.int32), ("edge_d", np.float64),
                         ("cell_i", np.int32), ("cell_d", np.float64), ("w_init", np.float64),
                         ("pis", np.float64), ("flux_raw", np.float64), ("ghost", np.float64),
                         ("grad", np.float64), ("umm", np.float64), ("sr_sum", np.float64),
                         ("gpu_counts", np.int32), ("gpu_w", np.float64),
                         ("wall_i", np.int32), ("nlog", np.int32)]:
            p = os.path.join(d, name + ".bin")
            if os.path.exists(p):
                out[name] = np.fromfile(p, dt)
        p = os.path.join(d, "drou_trace.bin")
        if os.path.exists(p):
            out["drou"] = np.fromfile(p, np.float64)
        out["w_at"] = {}
        for k in dump_at:
            p = os.path.join(d, f"w_at_{int(k)}.bin")
            if os.path.exists(p):
                out["w_at"][int(k)] = np.fromfile(p, np.float64).reshape(-1, 4)
        return out
    finally:
        if own:
            shutil.rmtree(d, ignore_errors=True)

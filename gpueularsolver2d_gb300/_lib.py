"""ctypes binding of ``libeuler2d.so`` -- the same C ABI a C/C++ caller links.

The library is built in-tree by ``gpueularsolver2d_gb300.build``.  There is no
fallback: if the library is missing, loading raises.
"""
from __future__ import annotations

import ctypes
import os

from . import build as _build

LIB_PATH = _build.LIB

E2D_FP64, E2D_FP32 = 0, 1
E2D_ORDER_FILE, E2D_ORDER_MORTON, E2D_ORDER_RCM = 0, 1, 2
E2D_LIMITER_REFERENCE, E2D_LIMITER_VENKAT, E2D_LIMITER_CELL_BARTH, E2D_LIMITER_CELL_VENKAT = 0, 1, 2, 3


class E2DError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"euler2d error {code}: {msg}")
        self.code = code


class Params(ctypes.Structure):
    """Mirror of ``e2d_params`` in include/euler2d.h."""
    _fields_ = [
        ("ma", ctypes.c_double), ("alpha_deg", ctypes.c_double), ("gamma", ctypes.c_double),
        ("pin", ctypes.c_double), ("tin", ctypes.c_double), ("cfl", ctypes.c_double),
        ("epsl", ctypes.c_double), ("maxstep", ctypes.c_int32), ("rk_stages", ctypes.c_int32),
        ("rk_coef", ctypes.c_double * 8), ("irs_eps", ctypes.c_double),
        ("irs_sweeps", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("dt_cap", ctypes.c_double), ("entropy_eps", ctypes.c_double),
        ("wall_box", ctypes.c_double), ("ordering", ctypes.c_int32),
        ("block_size", ctypes.c_int32), ("graph_iters", ctypes.c_int32),
        ("verbose", ctypes.c_int32), ("limiter_freeze", ctypes.c_int32),
        ("limiter", ctypes.c_int32), ("limiter_k", ctypes.c_double),
        ("limiter_freeze_resd", ctypes.c_double), ("global_dt", ctypes.c_int32),
        ("far_field_fix", ctypes.c_int32), ("first_order_iters", ctypes.c_int32),
        ("positivity_fix", ctypes.c_int32),
    ]


class MeshInfo(ctypes.Structure):
    _fields_ = [("ncell", ctypes.c_int32), ("nnode", ctypes.c_int32), ("nedge", ctypes.c_int32),
                ("nwall", ctypes.c_int32), ("nfar", ctypes.c_int32)]


class Integrals(ctypes.Structure):
    """Mirror of ``e2d_integrals`` in include/euler2d.h."""
    _fields_ = [(n, ctypes.c_double) for n in ("cl", "cd", "mass", "mass_flux_far", "mass_flux_wall")]

    def as_dict(self) -> dict:
        return {n: getattr(self, n) for n, _ in self._fields_}


_P = ctypes.c_void_p
_I = ctypes.c_int32
_D = ctypes.c_double
_PP = ctypes.POINTER(ctypes.c_void_p)
_PD = ctypes.POINTER(ctypes.c_double)
_PI = ctypes.POINTER(ctypes.c_int32)

# name -> (restype, argtypes); every symbol declared in include/euler2d.h
SIGNATURES = {
    "e2d_last_error": (ctypes.c_char_p, []),
    "e2d_version": (ctypes.c_char_p, []),
    "e2d_params_default": (_I, [ctypes.POINTER(Params)]),
    "e2d_input_read": (_I, [ctypes.c_char_p, ctypes.POINTER(Params)]),
    "e2d_mesh_read": (_I, [ctypes.c_char_p, _PP]),
    "e2d_mesh_write": (_I, [ctypes.c_char_p, _P]),
    "e2d_mesh_write_binary": (_I, [ctypes.c_char_p, _P]),
    "e2d_mesh_from_arrays": (_I, [_I, _I, _PD, _PD, _PI, _PP]),
    "e2d_mesh_ogrid_naca0012": (_I, [_I, _I, _D, _D, _D, ctypes.c_uint64, _PP]),
    "e2d_mesh_free": (None, [_P]),
    "e2d_mesh_info_get": (_I, [_P, _D, ctypes.POINTER(MeshInfo)]),
    "e2d_mesh_topology": (_I, [_P, _D, _PI, _PD, _PI, _PD]),
    "e2d_mesh_nodes": (_I, [_P, _PD, _PD, _PI]),
    "e2d_mesh_order": (_I, [_P, _I, _PI]),
    "e2d_solver_create": (_I, [_P, ctypes.POINTER(Params), _PP]),
    "e2d_solver_destroy": (None, [_P]),
    "e2d_solve": (_I, [_P, _I, _D, _PD, _PI]),
    "e2d_step": (_I, [_P, _I]),
    "e2d_progress": (_I, [_P, _PI, _PD]),
    "e2d_residual_history": (_I, [_P, _PD, _I, _PI]),
    "e2d_set_residual_norm": (_I, [_P, _D]),
    "e2d_get_residual_norm": (_I, [_P, _PD]),
    "e2d_get_state": (_I, [_P, _PD]),
    "e2d_set_state": (_I, [_P, _PD]),
    "e2d_forces": (_I, [_P, _PD, _PD]),
    "e2d_solver_integrals": (_I, [_P, ctypes.POINTER(Integrals)]),
    "e2d_state_integrals": (_I, [_P, ctypes.POINTER(Params), _PD, ctypes.POINTER(Integrals)]),
    "e2d_write_residual_plt": (_I, [_P, ctypes.c_char_p]),
    "e2d_write_field_plt": (_I, [_P, _P, ctypes.c_char_p]),
    "e2d_write_wall_cp_plt": (_I, [_P, _P, ctypes.c_char_p]),
    "e2d_get_params": (_I, [_P, ctypes.POINTER(Params)]),
    "e2d_set_precision": (_I, [_P, _I]),
    "e2d_last_device_ms": (_I, [_P, _PD]),
    "e2d_launches_per_iteration": (_I, [_P, _PI]),
    "e2d_profile_passes": (_I, [_P, _I, _PD, _PI]),
    "e2d_set_stream": (_I, [_P, _P]),
    "e2d_step_noalloc": (_I, [_I, _P, _P, _P, _P, ctypes.POINTER(Params), _I, _P, _P, _PD, _P]),
    "e2d_batch_create": (_I, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Params), _I, _PP]),
    "e2d_batch_destroy": (None, [_P]),
    "e2d_batch_step": (_I, [_P, _I]),
    "e2d_batch_solve": (_I, [_P, _I, _D, _PI]),
    "e2d_batch_info": (_I, [_P, _PI, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "e2d_batch_get_state": (_I, [_P, _I, _PD]),
    "e2d_batch_set_state": (_I, [_P, _I, _PD]),
    "e2d_batch_progress": (_I, [_P, _I, _PI, _PD, _PI]),
    "e2d_batch_residual_history": (_I, [_P, _I, _PD, _I, _PI]),
    "e2d_batch_forces": (_I, [_P, _I, _PD, _PD]),
    "e2d_batch_set_launch": (_I, [_P, _I, _I]),
    "e2d_batch_get_launch": (_I, [_P, _PI, _PI]),
    "e2d_batch_autotune": (_I, [_P, ctypes.c_char_p, _I, _PI, _PI, _PD]),
    "e2d_batch_create_tuned": (_I, [ctypes.POINTER(ctypes.c_void_p), ctypes.POINTER(Params), _I, ctypes.c_char_p, _I,
                                    _PP, _PI]),
    "e2d_batch_last_device_ms": (_I, [_P, _PD]),
    "e2d_batch_launches_per_iteration": (_I, [_P, _PI]),
}

_lib = None


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load libeuler2d.so (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        if not build_if_missing:
            raise OSError(f"{LIB_PATH} is missing; run gpueularsolver2d_gb300/build.py")
        _build.build()
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(rc: int) -> None:
    if rc != 0:
        raise E2DError(rc, load().e2d_last_error().decode())


class MLPConfig(ctypes.Structure):
    """Mirror of ``e2d_mlp_config`` in include/euler2d.h."""
    _fields_ = [("nhidden", ctypes.c_int32), ("batch", ctypes.c_int32), ("seed", ctypes.c_uint64),
                ("lr", ctypes.c_double), ("beta1", ctypes.c_double), ("beta2", ctypes.c_double),
                ("eps", ctypes.c_double)]


_PF = ctypes.POINTER(ctypes.c_float)
SIGNATURES.update({
    "e2d_mlp_config_default": (_I, [ctypes.POINTER(MLPConfig)]),
    "e2d_mlp_create": (_I, [ctypes.POINTER(MLPConfig), _PP]),
    "e2d_mlp_destroy": (None, [_P]),
    "e2d_mlp_param_count": (_I, [_P, ctypes.POINTER(ctypes.c_int64)]),
    "e2d_mlp_get_params": (_I, [_P, _PF]),
    "e2d_mlp_set_params": (_I, [_P, _PF]),
    "e2d_mlp_set_data": (_I, [_P, ctypes.c_int64, _PF, _PF]),
    "e2d_mlp_set_lr": (_I, [_P, _D]),
    "e2d_mlp_train": (_I, [_P, _I, _PD]),
    "e2d_mlp_forward": (_I, [_P, ctypes.c_int64, _PF, _PF]),
    "e2d_mlp_gradient": (_I, [_P, _PF, _PF, _PD, _PF]),
    "e2d_mlp_features": (_I, [_P, _D, _D, _D, ctypes.c_uint64, _D, _PF]),
    "e2d_wall_distance": (_I, [_P, _D, _PD]),
})

"""ctypes binding of libdgx.so (include/dgx.h).

The library is loaded from the package's parent directory, where ``build.py`` puts it.
There is no fallback: importing this module raises if the library is missing, and every
compute call raises ``DGXError`` when no sm_103 GPU is present.
"""

from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG_ROOT = Path(__file__).resolve().parent.parent
LIB_PATH = Path(os.environ.get("DGX_LIBRARY", PKG_ROOT / "libdgx.so"))

OK = 0
ERR_INVALID, ERR_RUNTIME, ERR_RANGE, ERR_CUDA, ERR_NONFINITE, ERR_TIMEOUT = -1, -2, -3, -4, -5, -6
BASIS_MONOMIAL, BASIS_DUBINER, BASIS_LEGENDRE = 0, 1, 2
EULER, NAVIER_STOKES = 0, 1
FP64, MIXED, DF64 = 0, 1, 2
BC_FAR_FIELD, BC_SLIP_WALL, BC_NO_SLIP_WALL, BC_PERIODIC = 0, 1, 2, 3

# every function include/dgx.h declares, with (restype, argtypes)
_vp, _dp, _ip, _cp = C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_char_p
SIGNATURES = {
    "dgx_last_error": (C.c_char_p, []),
    "dgx_version": (C.c_char_p, []),
    "dgx_mesh_create": (C.c_int, [C.c_int, _dp, C.c_int, _ip, C.c_int, C.POINTER(C.c_char_p), _ip,
                                  C.c_int, _ip, C.POINTER(_vp)]),
    "dgx_mesh_create_rectangle": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                            C.c_double, C.c_int, C.POINTER(_vp)]),
    "dgx_mesh_set_periodic": (C.c_int, [_vp, _cp, _cp]),
    "dgx_mesh_set_bc": (C.c_int, [_vp, _cp, C.c_int, _dp]),
    "dgx_mesh_info": (C.c_int, [_vp, _ip, _ip, _ip]),
    "dgx_mesh_interior_faces": (C.c_int, [_vp, _ip]),
    "dgx_mesh_boundary_faces": (C.c_int, [_vp, _ip]),
    "dgx_mesh_arrays": (C.c_int, [_vp, _ip, _dp, _ip]),
    "dgx_mesh_create_nv": (C.c_int, [C.c_int, C.c_int, _dp, C.c_int, _ip, C.c_int, C.POINTER(C.c_char_p), _ip,
                                     C.c_int, _ip, C.POINTER(_vp)]),
    "dgx_mesh_vertices_per_element": (C.c_int, [_vp, _ip]),
    "dgx_mesh_create_rectangle_quad": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double,
                                                 C.c_double, C.c_int, C.POINTER(_vp)]),
    "dgx_mesh_destroy": (None, [_vp]),
    "dgx_create": (C.c_int, [_vp, _vp, C.POINTER(_vp)]),
    "dgx_destroy": (None, [_vp]),
    "dgx_info": (C.c_int, [_vp, _ip, _ip, _ip, _ip]),
    "dgx_residual": (C.c_int, [_vp, _vp, _vp, _vp]),
    "dgx_apply_mass_inv": (C.c_int, [_vp, _vp, _vp, _vp]),
    "dgx_rhs": (C.c_int, [_vp, _vp, _vp, _vp]),
    "dgx_rk3_step": (C.c_int, [_vp, _vp, C.c_double, C.c_int, _vp]),
    "dgx_rk3_stage": (C.c_int, [_vp, _vp, _vp, _vp, C.c_double, C.c_int, _vp]),
    "dgx_max_cfl": (C.c_int, [_vp, _vp, C.c_double, _dp, _vp]),
    "dgx_density_range": (C.c_int, [_vp, _vp, _dp, _dp, _vp]),
    "dgx_has_nan": (C.c_int, [_vp, _vp, _ip, _vp]),
    "dgx_quad_points": (C.c_int, [_vp, _dp]),
    "dgx_quad_points_device": (C.c_int, [_vp, _vp, _vp]),
    "dgx_project": (C.c_int, [_vp, _vp, _vp, _vp]),
    "dgx_residual_host": (C.c_int, [_vp, _dp, _dp]),
    "dgx_rk3_step_host": (C.c_int, [_vp, _dp, C.c_double, C.c_int]),
    "dgx_rk3_step_static": (C.c_int, [_vp, _vp, C.c_double, C.c_int, _vp]),
    "dgx_apply_mass_inv_host": (C.c_int, [_vp, _dp, _dp]),
    "dgx_project_host": (C.c_int, [_vp, _dp, _dp]),
    "dgx_state_alloc": (C.c_int, [_vp, C.POINTER(_vp)]),
    "dgx_state_free": (None, [_vp]),
    "dgx_state_copy": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "dgx_monitor_host": (C.c_int, [_vp, _dp, C.c_double, _dp, _dp, _dp, _ip]),
    "dgx_residual_jvp": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "dgx_residual_vjp": (C.c_int, [_vp, _vp, _vp, _vp, _vp]),
    "dgx_rk3_step_tlm": (C.c_int, [_vp, _vp, _vp, C.c_double, C.c_int, _vp]),
    "dgx_rk3_step_adjoint": (C.c_int, [_vp, _vp, _vp, C.c_double, _vp]),
    "dgx_kinetic_energy": (C.c_int, [_vp, _vp, _dp, _vp, _vp]),
    "dgx_kinetic_energy_gradient": (C.c_int, [_vp, _vp, C.c_double, C.c_int, C.c_int, _dp, _vp, _vp]),
    "dgx_kinetic_energy_gradient_binomial": (C.c_int, [_vp, _vp, C.c_double, C.c_int, C.c_int, _dp, _vp,
                                                       C.POINTER(C.c_longlong), _vp]),
    "dgx_launch_shape": (C.c_int, [_vp, _ip, _ip, _ip]),
    "dgx_stage_tile": (C.c_int, [_vp, _ip, _ip]),
    "dgx_eval_points": (C.c_int, [_vp, C.c_int, _dp, _vp, _vp, _vp]),
    "dgx_step_status": (C.c_int, [_vp, _ip, _vp]),
    "dgx_batch_create": (C.c_int, [C.c_int, C.POINTER(_vp), _vp, C.POINTER(_vp)]),
    "dgx_batch_destroy": (None, [_vp]),
    "dgx_batch_info": (C.c_int, [_vp, C.c_int, _ip, _ip, C.POINTER(_vp)]),
    "dgx_batch_rk3_step": (C.c_int, [_vp, _dp, C.c_int, _vp]),
    "dgx_batch_launch_shape": (C.c_int, [_vp, _ip, _ip]),
    "dgx_batch_stage_form": (C.c_int, [_vp, _ip]),
}
STATIC_MAX_STATE = 1 << 20  # DGX_STATIC_MAX_STATE


class Params(C.Structure):
    _fields_ = [("order", C.c_int), ("basis", C.c_int), ("physics", C.c_int),
                ("precision", C.c_int), ("gamma", C.c_double), ("mu", C.c_double),
                ("prandtl", C.c_double), ("sigma0", C.c_double)]


class DGXError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{msg} (status {code})")
        self.code = code


class DGXInvalidArgument(DGXError, ValueError):
    pass


class DGXOutOfRange(DGXError, IndexError):
    pass


_lib = None


def load() -> C.CDLL:
    """Load libdgx.so and declare its signatures; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise ImportError(f"{LIB_PATH} not found: build it with "
                              f"`python {PKG_ROOT / 'build.py'}` (no CPU fallback exists)")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def check(code: int):
    """Turn a dgx status into the exception type dgfem would throw."""
    if code == OK:
        return
    msg = load().dgx_last_error().decode(errors="replace")
    if code == ERR_INVALID:
        raise DGXInvalidArgument(code, msg)
    if code == ERR_RANGE:
        raise DGXOutOfRange(code, msg)
    raise DGXError(code, msg)

"""ctypes loader for libxg (the C ABI in include/xg.h).

The library is built in-tree (xyst_gb300/_build/libxg.so) by
xyst_gb300/build.py.  There is no fallback: if the library is missing or fails
to load, every entry point raises.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

_i64 = C.c_int64
_i32 = C.c_int32
_dbl = C.c_double
_vp = C.c_void_p
_int = C.c_int

XG_OK = 0
STATUS = {0: "XG_OK", 1: "XG_ERR_ARG", 2: "XG_ERR_CUDA", 3: "XG_ERR_STATE", 4: "XG_ERR_BLOWUP",
          5: "XG_ERR_NOTCONV", 6: "XG_ERR_DEVICE", 7: "XG_ERR_HOST"}


class XgError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS.get(code, code)}: {msg}")
        self.code = code


class RiecgParams(C.Structure):
    _fields_ = [("gamma", _dbl), ("flux", _int), ("stab2", _int), ("stab2coef", _dbl),
                ("cfl", _dbl), ("const_dt", _dbl), ("precision", _int)]


class KozcgParams(C.Structure):
    _fields_ = [("gamma", _dbl), ("cfl", _dbl), ("const_dt", _dbl), ("fct", _int),
                ("ctau", _dbl), ("fctclip", _int), ("fctsys", _int), ("precision", _int)]


class ChocgParams(C.Structure):
    _fields_ = [("mu", _dbl), ("cfl", _dbl), ("const_dt", _dbl), ("flux", _int), ("stab", _int),
                ("stab2", _int), ("stab2coef", _dbl), ("rk", _int), ("ppc", _int),
                ("ptol", _dbl), ("pmaxit", _i64), ("pmixed", _int), ("pinner_tol", _dbl),
                ("pguard", _int)]


# name -> (restype, argtypes); every function of include/xg.h
SIGNATURES = {
    "xg_create": (_int, [_int, C.POINTER(_vp)]),
    "xg_destroy": (_int, [_vp]),
    "xg_last_error": (C.c_char_p, [_vp]),
    "xg_device_bytes": (_int, [_vp, C.POINTER(_i64)]),
    "xg_riecg_setup": (_int, [_vp, C.POINTER(RiecgParams), _i64, _vp, _vp,
                              _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _vp]),
    "xg_riecg_set_bc": (_int, [_vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _vp,
                               _i64, _vp, _vp]),
    "xg_riecg_set_state": (_int, [_vp, _vp, _dbl]),
    "xg_riecg_get_state": (_int, [_vp, _vp, _vp]),
    "xg_riecg_grad": (_int, [_vp, _vp, _vp]),
    "xg_riecg_rhs": (_int, [_vp, _vp, _vp, _vp]),
    "xg_riecg_rhs_coloured": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "xg_riecg_set_source": (_int, [_vp, _int, _vp]),
    "xg_riecg_bc": (_int, [_vp]),
    "xg_riecg_dt": (_int, [_vp, _vp]),
    "xg_riecg_stage": (_int, [_vp, _int, _dbl]),
    "xg_riecg_run": (_int, [_vp, _i64, _vp, _vp]),
    "xg_riecg_profile": (_int, [_vp, _int]),
    "xg_riecg_kernel_times": (_int, [_vp, _int, _vp, _vp, _vp, _vp]),
    "xg_riecg_dt_noalloc": (_int, [_vp, _vp, _i64, _dbl, _dbl, _dbl, _vp, _vp]),
    "xg_kozcg_setup": (_int, [_vp, C.POINTER(KozcgParams), _i64, _vp, _vp, _i64, _vp]),
    "xg_kozcg_set_bc": (_int, [_vp, _i64, _vp, _vp, _i64, _vp, _vp, _vp]),
    "xg_kozcg_set_state": (_int, [_vp, _vp, _dbl]),
    "xg_kozcg_get_state": (_int, [_vp, _vp, _vp]),
    "xg_kozcg_rhs": (_int, [_vp, _vp, _dbl, _vp]),
    "xg_kozcg_bc": (_int, [_vp]),
    "xg_kozcg_dt": (_int, [_vp, _vp]),
    "xg_kozcg_run": (_int, [_vp, _i64, _vp, _vp]),
    "xg_kozcg_step": (_int, [_vp, _dbl]),
    "xg_kozcg_set_source": (_int, [_vp, _int, _vp]),
    "xg_chocg_setup": (_int, [_vp, C.POINTER(ChocgParams), _i64, _vp, _vp, _i64, _vp, _vp,
                              _i64, _vp, _vp, _i64, _vp, _vp, _i64, _vp]),
    "xg_chocg_set_bc": (_int, [_vp, _i64, _vp, _vp, _vp, _i64, _vp, _vp, _i64, _vp, _i64, _vp,
                               _vp]),
    "xg_chocg_set_state": (_int, [_vp, _vp, _vp, _dbl]),
    "xg_chocg_get_state": (_int, [_vp, _vp, _vp, _vp]),
    "xg_chocg_init": (_int, [_vp, _vp]),
    "xg_chocg_run": (_int, [_vp, _i64, _vp, _vp, _vp]),
    "xg_chocg_set_theta": (_int, [_vp, _dbl, _i64, _vp, _int, _i64, _dbl]),
    "xg_chocg_momentum_its": (_int, [_vp, _vp]),
    "xg_chocg_fields": (_int, [_vp, _int, _vp]),
    "xg_chorin_div": (_int, [_vp, _vp, _vp, _vp, _dbl, _int, _vp]),
    "xg_chorin_grad": (_int, [_vp, _vp, _vp]),
    "xg_chorin_vgrad": (_int, [_vp, _vp, _vp]),
    "xg_chorin_flux": (_int, [_vp, _vp, _vp, _vp]),
    "xg_chorin_rhs": (_int, [_vp, _vp, _vp, _vp, _vp]),
    "xg_cg_setup": (_int, [_vp, _i64, _vp, _vp, _vp, _int]),
    "xg_cg_mult": (_int, [_vp, _vp, _vp]),
    "xg_cg_init": (_int, [_vp, _vp, _vp, _vp, _i64, _vp, _vp, _int, _int]),
    "xg_cg_solve": (_int, [_vp, _i64, _dbl, _vp, _vp, _vp, _vp]),
    "xg_cg_solve_mixed": (_int, [_vp, _i64, _dbl, _dbl, _i64, _vp, _vp, _vp, _vp, _vp]),
    "xg_cg_solution": (_int, [_vp, _vp]),
    "xg_cg_set_factor": (_int, [_vp, _vp, _dbl]),
    "xg_cg_precondition": (_int, [_vp, _vp, _vp]),
    "xg_cg_set_guard": (_int, [_vp, _int]),
    "xg_lpc_nparams": (_i64, []),
    "xg_lpc_create": (_int, [_vp, _int, C.POINTER(_vp)]),
    "xg_lpc_destroy": (_int, [_vp]),
    "xg_lpc_set_params": (_int, [_vp, _vp]),
    "xg_lpc_get_params": (_int, [_vp, _vp]),
    "xg_lpc_zero_grads": (_int, [_vp]),
    "xg_lpc_get_grads": (_int, [_vp, _vp]),
    "xg_lpc_grad": (_int, [_vp, _vp, _vp]),
    "xg_lpc_adam": (_int, [_vp, _dbl, _dbl, _dbl, _dbl]),
    "xg_lpc_last_error": (C.c_char_p, [_vp]),
    "xg_mesh_rcm": (_int, [_i64, _i64, _vp, _vp]),
    "xg_mesh_vol": (_int, [_i64, _vp, _i64, _vp, _vp]),
    "xg_mesh_edges": (_int, [_i64, _vp, _i64, _vp, _vp, _int, _i64, _vp, _vp, _vp]),
    "xg_mesh_bnorm": (_int, [_i64, _vp, _i64, _vp, _i64, _vp, _vp]),
    "xg_mesh_pressure_matrix": (_int, [_i64, _vp, _i64, _vp, _i64, _vp, _vp, _vp, _vp]),
}

_lib = None


def path() -> str:
    return _build.LIB


def load(build_if_missing: bool = True):
    """Load libxg, building it first when it is missing or stale."""
    global _lib
    if _lib is not None:
        return _lib
    if build_if_missing and not _build.up_to_date():
        _build.build()
    if not os.path.exists(_build.LIB):
        raise RuntimeError(f"libxg not built: {_build.LIB} missing")
    lib = C.CDLL(_build.LIB)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


def p(a):
    """Pointer to a numpy array's data (None passes NULL)."""
    return None if a is None else a.ctypes.data_as(_vp)


def f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def u64(a):
    return np.ascontiguousarray(a, dtype=np.uint64)


def i32(a):
    return np.ascontiguousarray(a, dtype=np.int32)


def u8(a):
    return np.ascontiguousarray(a, dtype=np.uint8)


class Context:
    """One device, one CUDA stream (xg_create)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = _vp()
        rc = self.lib.xg_create(device, C.byref(h))
        if rc != XG_OK:
            raise XgError(rc, f"xg_create({device}) failed (no CUDA device?)")
        self.h = h
        self.device = device

    def check(self, rc: int):
        if rc != XG_OK:
            raise XgError(rc, self.lib.xg_last_error(self.h).decode())

    def device_bytes(self) -> int:
        b = _i64()
        self.check(self.lib.xg_device_bytes(self.h, C.byref(b)))
        return int(b.value)

    def close(self):
        if getattr(self, "h", None):
            self.lib.xg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

"""ctypes binding of libomni3d_gb300.so (the C ABI declared in include/omni3d.h).

Loading fails loudly when the library has not been built: there is no fallback path.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB

OK = 0
ERR_ARG = -1
ERR_CUDA = -2
ERR_IO = -3
ERR_NOMEM = -4
ERR_STATE = -5
ERR_RANGE = -6
ERR_NUMERIC = -7

METHOD_PLAIN, METHOD_SELECT, METHOD_WEIGHTED = 0, 1, 2
METHOD_WEIGHTED_FIXED_BC, METHOD_SELECT_FIXED_BC, METHOD_MINI_CURL, METHOD_WEIGHTED_MINI_CURL = 3, 4, 5, 6
ENGINE_AUTO, ENGINE_LINES, ENGINE_BRICKS = 0, 1, 2
SOLVER_ANCHOR, SOLVER_SWEEP = 0, 1
GRAD_F32, GRAD_BF16 = 0, 1
GAUGE_NONE, GAUGE_POINT, GAUGE_MEAN = 0, 1, 2

_f = C.c_float
_d = C.c_double
_i = C.c_int
_ll = C.c_longlong
_fp = C.POINTER(C.c_float)
_vp = C.c_void_p


class Params(C.Structure):
    _fields_ = [("nx", _i), ("ny", _i), ("nz", _i), ("dx", _f), ("dy", _f), ("dz", _f), ("density", _f),
                ("line_spacing", _f), ("n_dirs", _i), ("dirs", _fp), ("max_iter", _i), ("threshold", _f),
                ("method", _i), ("solver", _i), ("grad_storage", _i), ("tol", _d), ("gauge", _i),
                ("ref_i", _i), ("ref_j", _i), ("ref_k", _i), ("seed_first_iteration", _i), ("device", _i),
                ("anchor_max_links", _ll), ("engine", _i), ("initial_guess", _i),
                ("sweep_fp64", _i), ("tile_width", _i), ("dir_group", _i), ("autotune", _i),
                ("deterministic", _i)]


class Stats(C.Structure):
    _fields_ = [("iterations", _i), ("rel_change", _d), ("n_lines", _ll), ("n_units", _ll), ("walk_errors", _ll),
                ("n_anchors", _ll), ("n_links", _ll), ("ms_geometry", _d), ("ms_setup", _d), ("ms_iterate", _d),
                ("ms_final", _d), ("ms_total", _d), ("ms_sweep", _d),
                ("kernel_launches", _ll), ("solver_used", _i), ("engine_used", _i), ("tile_width", _i),
                ("dir_group", _i)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


class FileParams(C.Structure):
    _fields_ = [("nx_org", _i), ("ny_org", _i), ("nz_org", _i), ("dx", _f), ("dy", _f), ("dz", _f),
                ("density", _f), ("scale", _f), ("line_spacing", _f), ("n_dirs", _i),
                ("dir_file", C.c_char * 1024), ("accel_dir", C.c_char * 1024), ("pressure_dir", C.c_char * 1024),
                ("n_iter", _i), ("threshold", _f), ("pref", _f), ("roi", _i * 6)]


# name -> (restype, argtypes); every symbol declared in include/omni3d.h
SIGNATURES = {
    "omni3d_default_params": (None, [C.POINTER(Params)]),
    "omni3d_create": (_i, [C.POINTER(Params), C.POINTER(_vp)]),
    "omni3d_destroy": (_i, [_vp]),
    "omni3d_last_error": (C.c_char_p, [_vp]),
    "omni3d_global_error": (C.c_char_p, []),
    "omni3d_set_stream": (_i, [_vp, _vp]),
    "omni3d_solve": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, C.POINTER(Stats)]),
    "omni3d_sweep": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i]),
    "omni3d_sweep_noalloc": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "omni3d_curl": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _i]),
    "omni3d_centre_integration": (_i, [_vp, _vp, _vp, _vp, C.c_double, _vp, _i]),
    "omni3d_gauge": (_i, [_vp, _vp, _vp, _ll, _i, _ll, _i]),
    "omni3d_adjoint": (_i, [_vp, _vp, _vp, _vp, _vp, _i]),
    "omni3d_geometry_info": (_i, [_vp, C.POINTER(_ll), C.POINTER(_ll), C.POINTER(_ll)]),
    "omni3d_line_table": (_i, [_vp, _vp, _ll]),
    "omni3d_line_steps": (_i, [_vp, _ll, _vp, _i]),
    "omni3d_batch_create": (_i, [_vp, _i, C.POINTER(_vp)]),
    "omni3d_batch_destroy": (_i, [_vp]),
    "omni3d_batch_last_error": (C.c_char_p, [_vp]),
    "omni3d_batch_solve": (_i, [_vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _i, C.POINTER(Stats)]),
    "omni3d_icosphere": (_i, [_i, _vp, _i]),
    "omni3d_read_directions": (_i, [C.c_char_p, _i, _vp]),
    "omni3d_read_params": (_i, [C.c_char_p, C.POINTER(FileParams)]),
    "omni3d_read_tecplot": (_i, [C.c_char_p, C.POINTER(FileParams), _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp, _vp,
                                 _vp]),
    "omni3d_bernoulli_face": (_i, [_i, _i, _i, _f, _f, _vp, _vp, _vp, _vp]),
    "omni3d_write_pressure": (_i, [C.c_char_p, _i, _i, _i, _vp, _vp, _vp, _vp, _vp]),
    "omni3d_write_curl": (_i, [C.c_char_p, _i, _i, _i, _vp, _vp, _vp, _vp]),
}

_lib = None


def lib() -> C.CDLL:
    """The loaded library.  Raises if it has not been built (no fallback exists)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError("libomni3d_gb300.so is not built (%s); run __graft_entry__.build() or "
                               "python -m omni3d.build" % LIB)
        L = C.CDLL(LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class Omni3DError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("omni3d error %d: %s" % (code, msg))
        self.code = code


def check(rc: int, ctx=None) -> int:
    if rc < 0:
        L = lib()
        msg = (L.omni3d_last_error(ctx) if ctx else L.omni3d_global_error()) or b""
        raise Omni3DError(rc, msg.decode(errors="replace"))
    return rc

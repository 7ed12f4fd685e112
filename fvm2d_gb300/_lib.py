"""ctypes binding of the C ABI declared in include/fvm_gpu.h.

The library is the in-tree ``_build/libfvm2d_gb300.so`` (``build.py``).  There
is no CPU fallback: if the library is missing, loading raises.
"""
from __future__ import annotations

import ctypes as C
import os

from .build import LIB as _LIB_MAIN
from .build import LIB_FP64FMA as _LIB_FP64FMA

# FVM_LIB_VARIANT=fp64fma loads the library whose FP64 kernels contract
# multiply-adds (for FP64 speed baselines); otherwise the main library
_VARIANT = os.environ.get("FVM_LIB_VARIANT", "")
if _VARIANT not in ("", "fp64fma"):
    raise RuntimeError(f"FVM_LIB_VARIANT={_VARIANT!r}: expected '' or 'fp64fma'")
LIB = _LIB_FP64FMA if _VARIANT == "fp64fma" else _LIB_MAIN

# codes (include/fvm_gpu.h, after src/param.h:97-142)
INVISCID, LAMINAR, TURBULENT = 1, 2, 3
ROE, KFVS, HLLC = 1, 2, 3
MEDIAN, BARTH = 1, 2
PT_INTERIOR, PT_SOLID, PT_OUTFLOW, PT_FARFIELD = 0, 3, 4, 5
FP64, FP32 = 0, 1

OK = 0
ERR_ARG, ERR_CUDA, ERR_NONPOSITIVE, ERR_ROE_SONIC, ERR_ZERO_FIRST_RES = 1, 2, 3, 4, 5
ERR_TIMEOUT, ERR_NOMEM, ERR_STATE, ERR_GEOMETRY, ERR_CAPACITY = 6, 7, 8, 9, 10
CHECKPOINTED = 11

_PARAM_DOUBLES = [
    "gamma", "gamma1", "gas_const", "pi", "prandtl", "prandtl_turb",
    "albada11", "albada12", "albada21", "albada22", "epsilon",
    "cb1", "cb2", "sigma_sa", "kolm", "cw1", "cw2", "cw3", "cv1", "cv2",
    "cv11", "cw31", "cw32", "kolm2", "cb2sig1", "cb2sig2",
    "mach_inf", "aoa_deg", "aoa", "rey", "cfl",
    "q_inf", "r_inf", "p_inf", "t_inf", "u_inf", "v_inf", "a_inf", "sconst", "nut_inf",
    "xref", "yref"]


class FvmParams(C.Structure):
    _fields_ = ([(n, C.c_int32) for n in ["iflow", "iflux", "ilimit", "vortex", "cell_type",
                                           "precision", "bugcompat", "reserved"]]
                + [(n, C.c_double) for n in _PARAM_DOUBLES]
                + [("airk", C.c_double * 3), ("birk", C.c_double * 3)])


_pd = C.POINTER(C.c_double)
_pi = C.POINTER(C.c_int32)


class FvmMesh(C.Structure):
    _fields_ = ([(n, C.c_int32) for n in ["np", "nt", "ne", "netot", "nsp", "nbe", "nswe1",
                                           "nswe2", "nffe1", "nffe2"]]
                + [("coord", _pd), ("elem", _pi), ("ptype", _pi), ("spts", _pi),
                   ("edge", _pi), ("iedge", _pi), ("beindx", _pi), ("ds", _pd),
                   ("elarea", _pd), ("cvarea", _pd), ("mcarea", _pd), ("drmin", _pd),
                   ("wd", _pd)])


class FvmGeom(C.Structure):
    _fields_ = [("mesh", FvmMesh), ("edge", _pi), ("edneigh", _pi), ("iedge", _pi),
                ("beindx", _pi), ("spts", _pi), ("ds", _pd), ("dsb", _pd), ("elarea", _pd),
                ("cvarea", _pd), ("mcarea", _pd), ("drmin", _pd), ("wd", _pd)]


class FvmBatchCaps(C.Structure):
    _fields_ = [("vertices", C.c_int64), ("meshes", C.c_int32), ("viscous", C.c_int32),
                ("blocks", C.c_int64), ("edge_entries", C.c_int64),
                ("boundary_entries", C.c_int64), ("tri_entries", C.c_int64),
                ("triangles", C.c_int64), ("edge_incidence", C.c_int64),
                ("tri_incidence", C.c_int64), ("all_incidence", C.c_int64),
                ("solid_edges", C.c_int64), ("max_slots", C.c_int32), ("max_tri", C.c_int32),
                ("grid", C.c_int32), ("max_tri2", C.c_int32), ("max_loc", C.c_int32),
                ("fused", C.c_int32), ("halo_entries", C.c_int64),
                ("halo_incidence", C.c_int64), ("grad_mode", C.c_int32),
                ("overlap", C.c_int32), ("pipe_groups", C.c_int32), ("pipe_stages", C.c_int32)]


# every function the header declares, with its signature
SIGNATURES = {
    "fvm_params_init": (C.c_int32, [C.POINTER(FvmParams), C.c_int32, C.c_double, C.c_double,
                                    C.c_double, C.c_double, C.c_int32, C.c_int32, C.c_int32,
                                    C.c_double, C.c_double, C.c_int32, C.c_double, C.c_int32,
                                    C.c_int32]),
    "fvm_gpu_create": (C.c_int32, [C.POINTER(FvmParams), C.POINTER(FvmMesh), C.POINTER(C.c_void_p)]),
    "fvm_gpu_destroy": (C.c_int32, [C.c_void_p]),
    "fvm_gpu_strerror": (C.c_char_p, [C.c_int32]),
    "fvm_gpu_set_state": (C.c_int32, [C.c_void_p, _pd, _pd, _pd, _pd, C.c_int32]),
    "fvm_gpu_get_state": (C.c_int32, [C.c_void_p, _pd, _pd, _pd, _pd, _pd, _pd]),
    "fvm_gpu_iterate": (C.c_int32, [C.c_void_p, C.c_int32, C.c_double, _pi, _pd, _pi, _pd,
                                    _pd, _pd, _pi]),
    "fvm_gpu_save_old": (C.c_int32, [C.c_void_p]),
    "fvm_gpu_time_step": (C.c_int32, [C.c_void_p]),
    "fvm_gpu_residu": (C.c_int32, [C.c_void_p]),
    "fvm_gpu_update": (C.c_int32, [C.c_void_p, C.c_int32]),
    "fvm_gpu_sa_model": (C.c_int32, [C.c_void_p]),
    "fvm_gpu_limitgrad": (C.c_int32, [C.c_void_p]),
    "fvm_gpu_check_positivity": (C.c_int32, [C.c_void_p, _pi]),
    "fvm_gpu_clcd": (C.c_int32, [C.c_void_p, _pd, _pd]),
    "fvm_gpu_conres": (C.c_int32, [C.c_void_p, C.c_int32, _pd, _pd, _pi]),
    "fvm_gpu_get_residual": (C.c_int32, [C.c_void_p, _pd]),
    "fvm_gpu_get_dt": (C.c_int32, [C.c_void_p, _pd]),
    "fvm_gpu_get_prim_old": (C.c_int32, [C.c_void_p, _pd]),
    "fvm_gpu_dtlength": (C.c_int32, [C.c_int32, C.c_int32, _pd, _pi, _pd, _pd]),
    "fvm_gpu_wall_dist": (C.c_int32, [C.c_int32, C.c_int32, _pd, _pi, _pi, C.c_int32, _pd]),
    "fvm_geom_build": (C.c_int32, [C.c_int32, C.c_int32, _pd, _pi, _pi, C.c_int32,
                                   C.POINTER(C.POINTER(FvmGeom))]),
    "fvm_geom_free": (C.c_int32, [C.POINTER(FvmGeom)]),
    "fvm_gpu_geom_build": (C.c_int32, [C.c_int32, C.c_int32, _pd, _pi, _pi, C.c_int32,
                                       C.POINTER(C.POINTER(FvmGeom))]),
    "fvm_batch_create": (C.c_int32, [C.c_int32, C.POINTER(FvmBatchCaps), C.POINTER(C.c_void_p)]),
    "fvm_batch_destroy": (C.c_int32, [C.c_void_p]),
    "fvm_batch_add": (C.c_int32, [C.c_void_p, C.POINTER(FvmParams), C.POINTER(FvmMesh), _pi]),
    "fvm_batch_remove": (C.c_int32, [C.c_void_p, C.c_int32]),
    "fvm_batch_set_state": (C.c_int32, [C.c_void_p, C.c_int32, _pd, _pd, _pd, _pd, C.c_int32]),
    "fvm_batch_get_state": (C.c_int32, [C.c_void_p, C.c_int32, _pd, _pd, _pd, _pd, _pd, _pd]),
    "fvm_batch_start": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_double]),
    "fvm_batch_step": (C.c_int32, [C.c_void_p, C.c_int32]),
    "fvm_batch_sync": (C.c_int32, [C.c_void_p]),
    "fvm_batch_poll": (C.c_int32, [C.c_void_p, C.c_int32, _pi, _pi, _pd, _pd, _pd, _pi, _pi]),
    "fvm_batch_history": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32, _pd, _pi,
                                      _pd, _pd, _pd]),
    "fvm_batch_history_depth": (C.c_int32, []),
    "fvm_batch_stream": (C.c_void_p, [C.c_void_p]),
    "fvm_batch_timing": (C.c_int32, [C.c_void_p, C.c_int32]),
    "fvm_batch_timing_read": (C.c_int32, [C.c_void_p, C.c_int32, C.c_char_p, _pd,
                                          C.POINTER(C.c_int64), _pi]),
    "fvm_batch_launch_count": (C.c_int64, [C.c_void_p]),
    "fvm_batch_test_wait_timeout": (C.c_int32, [C.c_void_p, C.c_int64]),
    "fvm_gpu_gradient": (C.c_int32, [C.c_void_p]),
    "fvm_gpu_shockind": (C.c_int32, [C.c_void_p]),
    "fvm_batch_tune": (C.c_int32, [C.c_void_p, C.c_int32, C.c_int32, _pd, _pi]),
    "fvm_batch_set_form": (C.c_int32, [C.c_void_p, C.c_int32]),
    "fvm_abi_sizes": (None, [C.POINTER(C.c_int64)]),
    "fvm_serve_create": (C.c_int32, [C.c_int32, C.c_void_p, C.c_int32, C.c_int32,
                                     C.POINTER(C.c_void_p)]),
    "fvm_serve_submit": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.c_double,
                                     C.c_int32, C.POINTER(C.c_int64)]),
    "fvm_serve_poll": (C.c_int32, [C.c_void_p, C.c_int64, _pi]),
    "fvm_serve_wait": (C.c_int32, [C.c_void_p, C.c_int64, C.c_double, _pi]),
    "fvm_serve_result": (C.c_int32, [C.c_void_p, C.c_int64, _pi, _pi, _pd, _pd, _pd, _pd, _pd]),
    "fvm_serve_state": (C.c_int32, [C.c_void_p, C.c_int64, _pd, _pd]),
    "fvm_serve_release": (C.c_int32, [C.c_void_p, C.c_int64]),
    "fvm_serve_checkpoint": (C.c_int32, [C.c_void_p, C.c_int64]),
    "fvm_serve_checkpoint_read": (C.c_int32, [C.c_void_p, C.c_int64, _pd, _pd, _pd, _pd, _pi]),
    "fvm_serve_resume": (C.c_int32, [C.c_void_p, C.POINTER(FvmParams), C.POINTER(FvmMesh),
                                     C.c_int32, C.c_double, _pd, _pd, _pd, _pd, C.c_int32,
                                     C.c_int32, C.POINTER(C.c_int64)]),
    "fvm_serve_stats": (C.c_int32, [C.c_void_p, C.POINTER(C.c_int64)]),
    "fvm_serve_times": (C.c_int32, [C.c_void_p, C.POINTER(C.c_double)]),
    "fvm_serve_destroy": (C.c_int32, [C.c_void_p]),
    "fvm_layout_stats": (C.c_int32, [C.POINTER(FvmMesh), C.POINTER(C.c_int64)]),
    "fvm_gpu_conres_noalloc": (C.c_int32, [C.c_void_p, C.c_void_p, C.c_int32, C.c_int32, _pd,
                                           _pd, _pd, _pi]),
    "fvm_batch_prepare": (C.c_int32, [C.POINTER(FvmParams), C.POINTER(FvmMesh),
                                      C.POINTER(C.c_void_p)]),
    "fvm_batch_add_prepared": (C.c_int32, [C.c_void_p, C.c_void_p, _pi]),
    "fvm_prepared_free": (C.c_int32, [C.c_void_p]),
    "fvm_prepared_bytes": (C.c_int64, [C.c_void_p, C.c_int32]),
}

_lib = None


class FvmError(RuntimeError):
    def __init__(self, status: int, what: str = ""):
        self.status = status
        msg = lib().fvm_gpu_strerror(status).decode() if _lib is not None else str(status)
        super().__init__(f"{what}: status {status} ({msg})" if what else f"status {status} ({msg})")


def lib():
    """Load the library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"{LIB} is missing: build it with fvm2d_gb300.build.build() "
                               "(there is no CPU fallback)")
        L = C.CDLL(LIB)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(status: int, what: str = "") -> None:
    if status != OK:
        raise FvmError(status, what)


def dptr(a):
    return a.ctypes.data_as(_pd) if a is not None else None


def iptr(a):
    return a.ctypes.data_as(_pi) if a is not None else None

"""ctypes binding of the C ABI declared in include/mcfd.h.

The shared library is ``libmcfd.so`` next to this file (built by
``pvcriemannsolvers_gb300.build``).  Loading fails loudly when it is missing:
there is no CPU fallback for any entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

LIB_PATH = Path(__file__).resolve().parent / "libmcfd.so"

# enum values of include/mcfd.h
OK = 0
ERR_ARGUMENT, ERR_MESH, ERR_CUDA, ERR_STATE, ERR_NOT_CONVERGED, ERR_UNSUPPORTED, ERR_NO_DEVICE, ERR_IO = range(1, 9)
EXACT, HLLC, AUSM, ROE, RUSANOV = range(5)
RIEMANN = {"exact": EXACT, "hllc": HLLC, "ausm": AUSM, "roe": ROE, "rusanov": RUSANOV}
BC_NONE, BC_INVISCID_WALL, BC_SUPERSONIC_INLET, BC_SUPERSONIC_OUTLET, BC_SUBSONIC_INLET, \
    BC_SUBSONIC_OUTLET, BC_SMART, BC_NO_SLIP_WALL = range(8)
INIT_AVERAGE, INIT_MAJORITY = 1, 2
STATE_CONSTANT, STATE_MOVING_SPLIT, STATE_OBLIQUE_SPLIT, STATE_TABLE = 0, 1, 2, 3
HEX8, TET4 = 0, 1
DGSEM, FR, MODAL = 0, 1, 2
SCHEME = {"dgsem": DGSEM, "fr": FR, "modal": MODAL}
FP64, MIXED = 0, 1
CONTRACTION = {"simt": 0, "tensor": 1}


class MeshDesc(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int64),
        ("xyz", C.POINTER(C.c_double)),
        ("n_cells", C.c_int64),
        ("cell_nodes", C.POINTER(C.c_int64)),
        ("cell_type", C.POINTER(C.c_int32)),
        ("n_faces", C.c_int64),
        ("face_cells", C.POINTER(C.c_int64)),
        ("face_sides", C.POINTER(C.c_int32)),
        ("face_group", C.POINTER(C.c_int32)),
        ("face_shift", C.POINTER(C.c_double)),
        ("cell_node_stride", C.c_int32),
    ]


class Options(C.Structure):
    _fields_ = [
        ("degree", C.c_int32),
        ("scheme", C.c_int32),
        ("riemann", C.c_int32),
        ("precision", C.c_int32),
        ("cfl", C.c_double),
        ("device", C.c_int32),
        ("limiter", C.c_int32),
        ("weno_w0", C.c_double),
        ("weno_eps", C.c_double),
        ("contraction", C.c_int32),
        ("shock_cells_fp64", C.c_int32),
        ("reserved", C.c_int32 * 2),
    ]


class BcState(C.Structure):
    _fields_ = [
        ("kind", C.c_int32),
        ("program", C.c_int32),
        ("axis", C.c_int32),
        ("reserved", C.c_int32),
        ("position", C.c_double),
        ("speed", C.c_double),
        ("a", C.c_double * 5),
        ("b", C.c_double * 5),
        ("normal", C.c_double * 3),
    ]


# every symbol include/mcfd.h declares, with (restype, argtypes)
_P = C.c_void_p
_D = C.POINTER(C.c_double)
SIGNATURES = {
    "mcfd_abi_version": (C.c_int, []),
    "mcfd_last_error": (C.c_char_p, [_P]),
    "mcfd_create": (C.c_int, [C.POINTER(MeshDesc), C.POINTER(Options), C.POINTER(_P)]),
    "mcfd_destroy": (C.c_int, [_P]),
    "mcfd_column_size": (C.c_int64, [_P]),
    "mcfd_set_bc": (C.c_int, [_P, C.c_int32, C.POINTER(BcState)]),
    "mcfd_set_time": (C.c_int, [_P, C.c_double]),
    "mcfd_bc_point_count": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_int64)]),
    "mcfd_bc_points": (C.c_int, [_P, C.c_int32, _D, C.c_int64]),
    "mcfd_set_bc_table": (C.c_int, [_P, C.c_int32, _D, C.c_int64]),
    "mcfd_set_solution": (C.c_int, [_P, _D, C.c_int64]),
    "mcfd_get_solution": (C.c_int, [_P, _D, C.c_int64]),
    "mcfd_residual": (C.c_int, [_P, _D, C.c_int64]),
    "mcfd_set_solution_device": (C.c_int, [_P, _P, C.c_int64]),
    "mcfd_get_solution_device": (C.c_int, [_P, _P, C.c_int64]),
    "mcfd_residual_device": (C.c_int, [_P, _P, C.c_int64]),
    "mcfd_residual_device_noalloc": (C.c_int, [_P, _P, _P, C.c_int64]),
    "mcfd_time_step": (C.c_int, [_P, C.c_double, C.c_int32, _D]),
    "mcfd_rk_step": (C.c_int, [_P, C.c_double, C.c_double, C.c_int32]),
    "mcfd_advance": (C.c_int, [_P, C.c_int32, C.c_double, C.c_int32, _D]),
    "mcfd_face_slot_count": (C.c_int64, [C.c_int64, C.POINTER(C.c_int32)]),
    "mcfd_build_faces": (C.c_int, [C.c_int64, _D, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                   C.c_int32, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.c_int32,
                                   C.POINTER(C.c_int32), _D, C.c_int64, C.POINTER(C.c_int64),
                                   C.POINTER(C.c_int32), C.POINTER(C.c_int32), _D, C.POINTER(C.c_int64)]),
    "mcfd_build_error": (C.c_char_p, []),
    "mcfd_build_faces_gpu": (C.c_int, [C.c_int32, C.c_int64, _D, C.c_int64, C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int32), C.c_int32, C.c_int64, C.POINTER(C.c_int64),
                                       C.POINTER(C.c_int32), C.c_int32, C.POINTER(C.c_int32), _D, C.c_int64,
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int32), C.POINTER(C.c_int32), _D,
                                       C.POINTER(C.c_int64)]),
    "mcfd_vtk_read": (C.c_int, [C.c_char_p, C.c_char_p, C.POINTER(C.c_void_p)]),
    "mcfd_vtk_mesh_sizes": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                      C.POINTER(C.c_int64)]),
    "mcfd_vtk_mesh_stride": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "mcfd_vtk_mesh_arrays": (C.c_int, [C.c_void_p, _D, C.POINTER(C.c_int64), C.POINTER(C.c_int32),
                                       C.POINTER(C.c_int64), C.POINTER(C.c_int32)]),
    "mcfd_vtk_mesh_destroy": (None, [C.c_void_p]),
    "mcfd_vtk_error": (C.c_char_p, []),
    "mcfd_hilbert_order": (C.c_int, [C.c_int64, _D, C.POINTER(C.c_int64)]),
    "mcfd_vtk_point_count": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "mcfd_vtk_sample": (C.c_int, [_P, _D, _D, C.POINTER(C.c_uint8), C.c_int64]),
    "mcfd_write_vtu": (C.c_int, [_P, C.c_char_p, C.c_char_p, C.c_int32]),
    "mcfd_write_vtu_arrays": (C.c_int, [C.c_char_p, C.c_char_p, C.c_int64, _D, _D, C.c_int64,
                                        C.POINTER(C.c_uint8), C.c_int32]),
    "mcfd_base64_encode": (C.c_int, [C.POINTER(C.c_uint8), C.c_int64, C.c_char_p, C.c_int64,
                                     C.POINTER(C.c_int64)]),
    "mcfd_gather_fields": (C.c_int, [_P, _P, C.c_int64]),
    "mcfd_scatter_fields": (C.c_int, [_P, _P, C.c_int64]),
    "mcfd_write_restart": (C.c_int, [_P, C.c_char_p, C.c_double]),
    "mcfd_read_restart": (C.c_int, [_P, C.c_char_p, _D]),
    "mcfd_ensemble_stream_begin": (C.c_int, [_P]),
    "mcfd_ensemble_stream_step": (C.c_int, [_P, C.POINTER(_D), C.POINTER(_D), C.c_int32, C.c_double, C.c_int32]),
    "mcfd_ensemble_stream_end": (C.c_int, [_P]),
    "mcfd_stream_begin": (C.c_int, [_P]),
    "mcfd_stream_step": (C.c_int, [_P, _D, _D, C.c_int64, C.c_double, C.c_int32, C.c_double, C.c_int32]),
    "mcfd_stream_end": (C.c_int, [_P]),
    "mcfd_set_stream": (C.c_int, [_P, _P]),
    "mcfd_synchronize": (C.c_int, [_P]),
    "mcfd_face_node_maps": (C.c_int, [_P, C.POINTER(C.c_int16), C.POINTER(C.c_int16)]),
    "mcfd_launch_count": (C.c_int64, [_P]),
    "mcfd_kernel_times": (C.c_int, [_P, C.c_int32, _D]),
    "mcfd_limit": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "mcfd_set_viscosity": (C.c_int, [_P, C.c_double, C.c_double, C.c_double]),
    "mcfd_get_viscosity": (C.c_int, [_P, _D, C.c_int64]),
    "mcfd_initial_limiter": (C.c_int, [_P, C.c_int32]),
    "mcfd_troubled_cells": (C.c_int, [_P, C.POINTER(C.c_int64)]),
    "mcfd_set_cases": (C.c_int, [_P, C.c_int32, C.POINTER(C.c_int64)]),
    "mcfd_case_times": (C.c_int, [_P, _D, _D, C.c_int32]),
    "mcfd_ensemble_create": (C.c_int, [C.POINTER(_P), C.c_int32, C.POINTER(_P)]),
    "mcfd_ensemble_advance": (C.c_int, [_P, C.c_int32, C.c_double, C.c_int32]),
    "mcfd_ensemble_destroy": (C.c_int, [_P]),
    "mcfd_ensemble_set_stream": (C.c_int, [_P, _P]),
    "mcfd_ensemble_last_error": (C.c_char_p, [_P]),
    "mcfd_autotune": (C.c_int, [_P, C.c_char_p, C.POINTER(C.c_int32)]),
    "mcfd_point_count": (C.c_int64, [_P]),
    "mcfd_points": (C.c_int, [_P, _D, C.c_int64]),
    "mcfd_project": (C.c_int, [_P, _D, C.c_int64]),
    "mcfd_probe_flux": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_int64, _P, _P, _P, _P,
                                  C.POINTER(C.c_uint32)]),
    "mcfd_probe_numerics": (C.c_int, [C.c_int32, C.c_int32, C.c_int64, _P, _P]),
}
PROBE_RCP, PROBE_RCP_SIGNED, PROBE_SQRT_SEEDED, PROBE_F64_TO_F32, PROBE_F32_TO_F64, \
    PROBE_CUDA_RCP, PROBE_CUDA_SQRT, PROBE_CUDA_F64_TO_F32, PROBE_CUDA_F32_TO_F64, PROBE_RCP1, \
    PROBE_ROOT7, PROBE_ROOT7_OVER_X, PROBE_POW_NEG_GAMMA, PROBE_CUDA_POW_ROOT7, \
    PROBE_CUDA_POW_NEG_GAMMA = range(15)
LIMITER = {"none": 0, "lazy": 1, "detect_lazy": 2, "eigen": 3}

_lib = None


def load() -> C.CDLL:
    """Load libmcfd.so (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise RuntimeError(
                f"{LIB_PATH} is missing: build it with "
                "`python -c 'import __graft_entry__ as g; g.build()'`")
        lib = C.CDLL(str(LIB_PATH))
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


class McfdError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"mcfd error {code}: {msg}")
        self.code = code


def dptr(a: np.ndarray):
    return a.ctypes.data_as(_D)


def check(code: int, handle=None) -> None:
    if code != OK:
        msg = load().mcfd_last_error(handle)
        raise McfdError(code, msg.decode() if msg else "")

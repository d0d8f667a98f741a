"""ctypes binding of ``libfdp.so`` (include/fdp.h, fdp_prep.h, fdp_io.h, fdp_edge.h).

The library is built in-tree by :mod:`fdporo.build`; loading fails loudly if
it is missing -- there is no CPU fallback for the time-stepping path.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from .build import LIB_PATH, build

FDP_OK = 0
FDP_ERR_ARG = -1
FDP_ERR_CUDA = -2
FDP_ERR_ALLOC = -3
FDP_ERR_STATE = -4
FDP_ERR_UNSUPPORTED = -5
FDP_ERR_DEVICE = -6
FDP_BATCH_SHOTS = -1
FDP_F32 = 4
FDP_F64 = 8

FDP_REC_TLV = 1
FDP_REC_TLQ = 2
FDP_REC_TLP = 4
FDP_REC_VALUES = 10

# enum fdp_field_id (include/fdp.h), names as in the reference's modules
FIELD_NAMES = [
    "UM", "WM", "QX", "QZ", "TXX", "TZZ", "TXZ", "PRES",
    "PZXL", "PZXH", "PXXL", "PXXH", "OXXL", "OXXH", "PXZH", "PZZH", "OZZH",
    "RXXL", "RXXH", "SXXL", "SXXH", "RZXL", "RZXH", "GXXL", "GXXH", "HXXL", "HXXH",
    "GZXL", "GZXH", "RXZH", "GXZH", "RZZH", "SZZH", "GZZH", "HZZH",
    "SZ_U", "SZ_W", "SZ_QX", "SZ_QZ",
    "QXP", "QZP",
]
FIELD_ID = {n: i for i, n in enumerate(FIELD_NAMES)}
WAVEFIELD = FIELD_NAMES[:8]
MEMORY_VARS = FIELD_NAMES[8:35]
HISTORY = FIELD_NAMES[35:39]

# the 24 PML profiles in fdp_set_pml order (ppml.F90:60-83)
PROFILE_NAMES = [
    "ODA_XL", "ODB_XL", "ODC_XL", "ODD_XL", "ODA_XH", "ODB_XH", "ODC_XH", "ODD_XH",
    "ODA_ZH", "ODB_ZH", "ODC_ZH", "ODD_ZH",
    "ODA2_XL", "ODB2_XL", "ODC2_XL", "ODD2_XL", "ODA2_XH", "ODB2_XH", "ODC2_XH", "ODD2_XH",
    "ODA2_ZH", "ODB2_ZH", "ODC2_ZH", "ODD2_ZH",
]


class fdp_grid(C.Structure):
    _fields_ = [
        ("mx", C.c_int32), ("mz", C.c_int32), ("tpml", C.c_int32), ("stress_imaging", C.c_int32),
        ("lin_x", C.c_int32), ("lin_z", C.c_int32), ("precision", C.c_int32), ("device", C.c_int32),
        ("h", C.c_double), ("dt", C.c_double), ("tau_eps", C.c_double),
    ]


# every symbol the headers declare, with (restype, argtypes)
_VP = C.c_void_p
_I32 = C.c_int32
_PI32 = C.POINTER(C.c_int32)
_D = C.c_double
_PD = C.POINTER(C.c_double)
SIGNATURES = {
    "fdp_create": (C.c_int, [C.POINTER(fdp_grid), C.POINTER(_VP)]),
    "fdp_set_medium": (C.c_int, [_VP, _PI32, _I32, _I32, _I32, _VP]),
    "fdp_share_medium": (C.c_int, [_VP, _VP]),
    "fdp_diag_wait_timeout": (C.c_int, [_VP, _I32]),
    "fdp_set_pml": (C.c_int, [_VP, C.POINTER(_VP)]),
    "fdp_set_pml_arrays": (C.c_int, [_VP] + [_VP] * 24),
    "fdp_set_bottom_nr": (C.c_int, [_VP, _VP]),
    "fdp_set_source": (C.c_int, [_VP, _VP, _I32]),
    "fdp_set_receivers": (C.c_int, [_VP, _PI32, _PI32, _PI32, _PI32, _I32, _I32]),
    "fdp_run": (C.c_int, [_VP, _I32, _I32]),
    "fdp_prepare_run": (C.c_int, [_VP, _I32]),
    "fdp_get_receivers": (C.c_int, [_VP, _I32, _I32, _VP]),
    "fdp_get_snapshot": (C.c_int, [_VP, _I32, _VP]),
    "fdp_field_bounds": (C.c_int, [_VP, _I32, _PI32]),
    "fdp_get_field": (C.c_int, [_VP, _I32, _VP]),
    "fdp_set_field": (C.c_int, [_VP, _I32, _VP]),
    "fdp_synchronize": (C.c_int, [_VP]),
    "fdp_kernel_launches": (C.c_int64, [_VP]),
    "fdp_get_stream": (C.c_int, [_VP, C.POINTER(_VP)]),
    "fdp_medium_info": (C.c_int, [_VP, _PI32, _PI32, _PI32]),
    "fdp_core_info": (C.c_int, [_VP, _PI32]),
    "fdp_march_info": (C.c_int, [_VP, _PI32, _PI32]),
    "fdp_profile_run": (C.c_int, [_VP, _I32, _I32, _PD, C.POINTER(C.c_int64)]),
    "fdp_last_error": (C.c_char_p, [_VP]),
    "fdp_receivers_noalloc": (C.c_int, [_I32, _VP, _VP, _VP, _VP, _VP, _VP, _I32, _I32, _I32, _I32, _VP, _I32,
                                        _I32, _D, _I32, _VP, _VP]),
    "fdp_destroy": (None, [_VP]),
    "fdp_batch_create": (C.c_int, [C.POINTER(_VP), _I32, C.POINTER(_VP)]),
    "fdp_batch_run": (C.c_int, [_VP, _I32, _I32]),
    "fdp_batch_set_shape": (C.c_int, [_VP, _I32, _I32]),
    "fdp_batch_get_shape": (C.c_int, [_VP, _PI32, _PI32]),
    "fdp_batch_synchronize": (C.c_int, [_VP]),
    "fdp_batch_kernel_launches": (C.c_int64, [_VP]),
    "fdp_batch_get_stream": (C.c_int, [_VP, C.POINTER(_VP)]),
    "fdp_batch_last_error": (C.c_char_p, [_VP]),
    "fdp_batch_destroy": (None, [_VP]),
    "fdp_edge_create": (C.c_int, [_I32, C.POINTER(C.c_float), C.c_uint64, C.POINTER(_VP)]),
    "fdp_edge_set_output": (C.c_int, [_VP, _I32]),
    "fdp_edge_get_params": (C.c_int, [_VP, C.POINTER(C.c_float)]),
    "fdp_edge_set_params": (C.c_int, [_VP, C.POINTER(C.c_float)]),
    "fdp_edge_get_scale": (C.c_int, [_VP, C.POINTER(C.c_float)]),
    "fdp_edge_set_scale": (C.c_int, [_VP, C.POINTER(C.c_float)]),
    "fdp_edge_forward": (C.c_int, [_VP, _I32, _PI32, C.POINTER(C.c_float), C.POINTER(C.c_float)]),
    "fdp_edge_gradients": (C.c_int, [_VP, _I32, _PI32, C.POINTER(C.c_float), C.POINTER(C.c_float),
                                     C.POINTER(C.c_float), _PD]),
    "fdp_edge_train_batch": (C.c_int, [_VP, _I32, _PI32, C.POINTER(C.c_float), C.POINTER(C.c_float), C.c_float,
                                       _PD]),
    "fdp_edge_train_level": (C.c_int, [_VP, _VP, _VP, _I32, _I32, C.c_float, _I32, _PD]),
    "fdp_edge_attach": (C.c_int, [_VP, _VP]),
    "fdp_edge_last_error": (C.c_char_p, [_VP]),
    "fdp_edge_destroy": (None, [_VP]),
    "fdp_prep_velocities": (C.c_int, [_I32, _D, _D, _D, _D, _D, _D, _D, _PD, _PD, _PD]),
    "fdp_prep_scale_table": (C.c_int, [_I32, _I32, _D, _D, _VP]),
    "fdp_prep_expand_jm": (C.c_int, [_I32, _I32, _I32, _I32, _PI32, _PI32]),
    "fdp_prep_pml": (C.c_int, [_I32, _I32, _I32, _I32, _I32, _D, _D, _D, _D, _D, _D, _D, _PI32, _I32, _VP,
                               C.POINTER(_VP)]),
    "fdp_prep_bottom_nr": (C.c_int, [_I32, _I32, _I32, _I32, _I32, _D, _D, _D, _D, _D, _D, _PI32, _I32, _VP, _VP]),
    "fdp_prep_source": (C.c_int, [_I32, _I32, _VP, _VP, _I32, _D, _D, _I32, _D, _VP]),
    "fdp_io_format_e": (C.c_int, [_D, _I32, _I32, C.c_char_p]),
    "fdp_io_namelist_get": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_char_p, C.c_size_t]),
    "fdp_io_read_record": (C.c_int, [C.c_char_p, C.c_int64, _VP, C.c_int64, C.POINTER(C.c_int64)]),
    "fdp_io_append_record": (C.c_int, [C.c_char_p, _VP, C.c_int64]),
}

_lib: C.CDLL | None = None


def lib_path() -> Path:
    return LIB_PATH


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads libfdp.so (building it first if it is absent and allowed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if not build_if_missing:
            raise RuntimeError(f"{LIB_PATH} is missing; run fdporo.build.build()")
        build()
    lib = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class FdpError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"fdp error {code}: {msg}")
        self.code = code

"""ctypes binding of libmpsq.so (the C ABI declared in include/mpsq.h).

Loading fails loudly when the library has not been built: there is no CPU fallback for any
compute entry point.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

from . import build as _build

MAX_SPECIES = 16
FP32, FP64 = 0, 1
CELL, BULK = 0, 1
WEIGHT_UNIT, WEIGHT_NEUTRON, WEIGHT_XRAY = 1, 2, 3
FF_MP_SQOM, FF_STANDARD = 0, 1
OPT_GRAPH, OPT_SPREAD, OPT_XROWS, OPT_LANES, OPT_ZSLAB, OPT_REPRODUCIBLE = 1, 2, 3, 4, 5, 6

ERR_NAMES = {0: "OK", 1: "ERR_ARG", 2: "ERR_ALLOC", 3: "ERR_CUDA", 4: "ERR_CUFFT",
             5: "ERR_STATE", 6: "ERR_DEVICE"}

# Every extern "C" symbol include/mpsq.h declares (checked by the CPU test suite).
EXPORTS = [
    "finufft2d1", "finufft3d1", "finufftf2d1", "finufftf3d1", "finufft2d1_", "finufft3d1_",
    "mpsq_nufft_makeplan", "mpsq_nufft_setpts", "mpsq_nufft_execute", "mpsq_nufft_destroy",
    "mpsq_nufft_info", "mpsq_nufft_check_error",
    "mpsq_job_create", "mpsq_job_destroy", "mpsq_job_estimate_bytes", "mpsq_job_set_frames",
    "mpsq_job_set_frames_on",
    "mpsq_job_set_cell_index", "mpsq_job_transform", "mpsq_job_amplitudes", "mpsq_job_sq_total",
    "mpsq_job_sqw_econst", "mpsq_job_sqw_dispersion", "mpsq_job_sqw_econst_pair",
    "mpsq_job_sqw_dispersion_pair", "mpsq_job_iqt", "mpsq_job_iqt_dispersion",
    "mpsq_job_sqw_gauss", "mpsq_job_sync", "mpsq_job_info", "mpsq_job_set_option",
    "mpsq_job_get_option", "mpsq_job_autotune", "mpsq_job_set_q_slab",
    "mpsq_job_profile", "mpsq_job_stage_ms", "mpsq_job_radial_hist", "mpsq_last_error",
    "mpsq_version", "mpsq_launch_count",
    "mpsq_nufft2d1_noalloc", "mpsq_speckle_filter", "mpsq_job_transform_onephonon",
]


class JobDesc(C.Structure):
    """Mirror of mpsq_job_desc."""
    _fields_ = [
        ("ndim", C.c_int32),
        ("precision", C.c_int32),
        ("eps", C.c_double),
        ("n_modes", C.c_int64 * 3),
        ("input_method", C.c_int32),
        ("phase_rounding", C.c_int32),
        ("axis", (C.c_double * 3) * 3),
        ("tpe", C.c_double * 3),
        ("centre", C.c_double * 3),
        ("use_range", C.c_int32),
        ("pos_min", C.c_double * 3),
        ("pos_max", C.c_double * 3),
        ("eps_x", C.c_double),
        ("bulk_nsuper1", C.c_int32),
        ("n_row", C.c_int32 * 3),
        ("q_center", C.c_double * 3),
        ("spatial_window", C.c_int32),
        ("n_species", C.c_int32),
        ("species_offset", C.c_int64 * (MAX_SPECIES + 1)),
        ("mask", C.c_int32 * MAX_SPECIES),
        ("weight_mode", C.c_int32),
        ("b_coh", C.c_double * MAX_SPECIES),
        ("xff", (C.c_double * 9) * MAX_SPECIES),
        ("ff_convention", C.c_int32),
        ("qphys_origin", C.c_double * 3),
        ("qphys_step", (C.c_double * 3) * 3),
        ("qphys_extra_sq", C.c_double),
        ("n_atoms_frame", C.c_int64),
        ("n_frames", C.c_int32),
        ("store_species", C.c_int32),
        ("no_pack", C.c_int32),
        ("no_pruned_fft", C.c_int32),
        ("stream_ordered", C.c_int32),
        ("q_slab", C.c_int64),
    ]


_lib = None


def lib_path() -> Path:
    return _build.LIB


def load(build_if_missing: bool = True) -> C.CDLL:
    """Loads libmpsq.so (building it first if requested); raises if unavailable."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path()
    if not path.exists() or (build_if_missing and not _build.up_to_date()):
        if not build_if_missing:
            raise RuntimeError(f"libmpsq.so not built at {path}")
        _build.build()
    lib = C.CDLL(str(path))
    vp, i64, i32, dbl = C.c_void_p, C.c_int64, C.c_int32, C.c_double
    sig = {
        "finufft2d1": (C.c_int, [i64, vp, vp, vp, C.c_int, dbl, i64, i64, vp, vp]),
        "finufft3d1": (C.c_int, [i64, vp, vp, vp, vp, C.c_int, dbl, i64, i64, i64, vp, vp]),
        "finufftf2d1": (C.c_int, [i64, vp, vp, vp, C.c_int, C.c_float, i64, i64, vp, vp]),
        "finufftf3d1": (C.c_int, [i64, vp, vp, vp, vp, C.c_int, C.c_float, i64, i64, i64, vp, vp]),
        "finufft2d1_": (None, [vp] * 11),
        "finufft3d1_": (None, [vp] * 13),
        "mpsq_nufft_makeplan": (C.c_int, [C.c_int, vp, C.c_int, C.c_int, dbl, C.c_int, vp, vp]),
        "mpsq_nufft_setpts": (C.c_int, [vp, i64, vp, vp, vp]),
        "mpsq_nufft_execute": (C.c_int, [vp, vp, vp]),
        "mpsq_nufft_destroy": (C.c_int, [vp]),
        "mpsq_nufft_info": (C.c_int, [vp, vp, vp]),
        "mpsq_nufft_check_error": (C.c_int, [vp]),
        "mpsq_job_create": (C.c_int, [vp, vp, vp]),
        "mpsq_job_destroy": (C.c_int, [vp]),
        "mpsq_job_estimate_bytes": (C.c_int, [vp, vp]),
        "mpsq_job_set_frames": (C.c_int, [vp, vp, i32, i32, C.c_int]),
        "mpsq_job_set_frames_on": (C.c_int, [vp, vp, i32, i32, C.c_int, vp]),
        "mpsq_job_set_cell_index": (C.c_int, [vp, vp, C.c_int]),
        "mpsq_job_transform": (C.c_int, [vp, i32, i32]),
        "mpsq_job_amplitudes": (C.c_int, [vp, vp]),
        "mpsq_job_sq_total": (C.c_int, [vp, dbl, vp, C.c_int]),
        "mpsq_job_sqw_econst": (C.c_int, [vp, i32, vp, i32, vp, dbl, vp, C.c_int]),
        "mpsq_job_sqw_dispersion": (C.c_int, [vp, i32, vp, i32, vp, i32, vp, dbl, vp, C.c_int]),
        "mpsq_job_sqw_gauss": (C.c_int, [vp, dbl, i32, vp, dbl, vp, C.c_int]),
        "mpsq_job_sqw_econst_pair": (C.c_int, [vp, i32, vp, i32, i32, i32, dbl, vp, C.c_int]),
        "mpsq_job_sqw_dispersion_pair": (C.c_int, [vp, i32, vp, i32, vp, i32, i32, i32, dbl, vp, C.c_int]),
        "mpsq_job_iqt": (C.c_int, [vp, i32, i32, vp, dbl, vp, C.c_int]),
        "mpsq_job_iqt_dispersion": (C.c_int, [vp, i32, i32, vp, vp, dbl, vp, C.c_int]),
        "mpsq_job_sync": (C.c_int, [vp]),
        "mpsq_job_info": (C.c_int, [vp, vp, vp, vp, vp, vp]),
        "mpsq_job_set_option": (C.c_int, [vp, C.c_int, C.c_int]),
        "mpsq_job_get_option": (C.c_int, [vp, C.c_int, vp]),
        "mpsq_job_autotune": (C.c_int, [vp, i32, i32, C.c_char_p, vp, vp]),
        "mpsq_job_set_q_slab": (C.c_int, [vp, i64]),
        "mpsq_job_profile": (C.c_int, [vp, C.c_int]),
        "mpsq_job_stage_ms": (C.c_int, [vp, vp, vp, C.c_int]),
        "mpsq_job_radial_hist": (C.c_int, [vp, vp, vp, dbl, dbl, i32, dbl, vp, C.c_int]),
        "mpsq_last_error": (C.c_char_p, []),
        "mpsq_version": (C.c_char_p, []),
        "mpsq_launch_count": (i64, []),
        "mpsq_nufft2d1_noalloc": (C.c_int, [i64, vp, vp, vp, C.c_int, dbl, i64, i64, vp, vp]),
        "mpsq_speckle_filter": (C.c_int, [vp, i64, i64, C.c_float, i32, C.c_float, i32, vp]),
        "mpsq_job_transform_onephonon": (C.c_int, [vp, i32, i32, i32, i32, C.c_float, C.c_float, vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _lib = lib
    return lib


class MpsqError(RuntimeError):
    def __init__(self, code: int, where: str):
        msg = load().mpsq_last_error().decode(errors="replace")
        super().__init__(f"{where}: {ERR_NAMES.get(code, code)}: {msg}")
        self.code = code


def check(code: int, where: str) -> None:
    if code != 0:
        raise MpsqError(code, where)


def ptr(a) -> int:
    """Address of a numpy array / torch tensor buffer (host or device)."""
    if a is None:
        return 0
    if hasattr(a, "data_ptr"):
        return int(a.data_ptr())
    return int(a.ctypes.data)

"""ctypes binding of libqsfgpu.so (include/qsf_gpu.h).

The shared library is built in-tree by qsf_gb300/build.py.  There is no fallback:
if the library is missing or fails to load, every entry point raises.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# QSF_LIB selects another build of the library (the autotuner's candidate builds under
# qsf_gb300/_build/); by default the in-tree qsf_gb300/libqsfgpu.so
LIB_PATH = os.environ.get("QSF_LIB") or os.path.join(HERE, "libqsfgpu.so")

QSF_OK = 0
ERRORS = {1: "EINVAL", 2: "ENOMEM", 3: "ECUDA", 4: "ETIMEDOUT", 5: "ENUMERIC", 6: "ESTATE", 7: "EBUSY",
          8: "ECANCELED"}
MAX_BORDERS = 16


class QsfError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: QSF_{ERRORS.get(code, code)}: {msg}")
        self.code = code


class GridDesc(ctypes.Structure):
    _fields_ = [
        ("dim", ctypes.c_int),
        ("n", ctypes.c_int64 * 3),
        ("dx", ctypes.c_double * 3),
        ("nCAP", ctypes.c_int64),
        ("potential", ctypes.c_int),
        ("Ncharge", ctypes.c_double),
        ("Echarge", ctypes.c_double),
        ("Nsoft", ctypes.c_double),
        ("Esoft", ctypes.c_double),
        ("gauge", ctypes.c_int),
        ("n_fields", ctypes.c_int),
        ("p_axis_swap", ctypes.c_int),
        ("border_nodes", ctypes.c_int64 * 4),
        ("free_axes", ctypes.c_int),
        ("multi_region", ctypes.c_int),
        ("absorber", ctypes.c_int),
        ("mask_dt", ctypes.c_double),
    ]


class Request(ctypes.Structure):
    _fields_ = [
        ("grid", GridDesc),
        ("mode", ctypes.c_int),
        ("dt", ctypes.c_double),
        ("nsteps", ctypes.c_int64),
        ("coupling", ctypes.POINTER(ctypes.c_double)),
        ("psi0", ctypes.POINTER(ctypes.c_double)),
        ("obs", ctypes.c_uint32),
        ("nborders", ctypes.c_int),
        ("border_types", ctypes.c_int * MAX_BORDERS),
        ("box_size", ctypes.c_int64),
    ]


class Result(ctypes.Structure):
    _fields_ = [
        ("status", ctypes.c_int),
        ("steps", ctypes.c_int64),
        ("final_norm", ctypes.c_double),
        ("yield_", ctypes.c_double),
        ("final_epot", ctypes.c_double),
        ("flux_integral", ctypes.c_double * MAX_BORDERS),
        ("queue_s", ctypes.c_double),
        ("latency_s", ctypes.c_double),
    ]


class ServerConfig(ctypes.Structure):
    _fields_ = [
        ("max_slots", ctypes.c_int),
        ("hbm_reserve_gb", ctypes.c_double),
        ("steps_per_round", ctypes.c_int64),
        ("queue_capacity", ctypes.c_int),
    ]


class ServerStats(ctypes.Structure):
    _fields_ = [
        ("submitted", ctypes.c_int64),
        ("admitted", ctypes.c_int64),
        ("completed", ctypes.c_int64),
        ("queued", ctypes.c_int64),
        ("in_flight", ctypes.c_int64),
        ("grid_point_steps", ctypes.c_double),
    ]


class StepDesc(ctypes.Structure):
    _fields_ = [
        ("mode", ctypes.c_int),
        ("dt", ctypes.c_double),
        ("nsteps", ctypes.c_int64),
        ("coupling", ctypes.POINTER(ctypes.c_double)),
        ("obs", ctypes.c_uint32),
        ("normalize", ctypes.c_int),
        ("nborders", ctypes.c_int),
        ("border_types", ctypes.c_int * MAX_BORDERS),
        ("box_size", ctypes.c_int64),
        ("state_accuracy", ctypes.c_double),
        ("last_energy", ctypes.c_double),
        ("energy_after_normalize", ctypes.c_int),
        ("kernel_ms", ctypes.POINTER(ctypes.c_float)),
        ("kernel_launches", ctypes.POINTER(ctypes.c_int64)),
        ("substeps", ctypes.c_int),
        ("ekin_interval", ctypes.c_int),
    ]


class DumpFormat(ctypes.Structure):
    _fields_ = [
        ("rep", ctypes.c_int),
        ("complex_values", ctypes.c_int),
        ("downscale", ctypes.c_int64),
        ("evo_backup", ctypes.c_int),
    ]


KERNEL_KINDS = ["tables", "row_open", "axis_fwd", "axis_fpi", "axis_inv", "row_close", "axis_ekin", "finalize",
                "line_step"]


_lib = None


def lib():
    """Load libqsfgpu.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"{LIB_PATH} is missing: build it with `python -m qsf_gb300.build`")
    L = ctypes.CDLL(LIB_PATH)
    vp = ctypes.c_void_p
    dp = ctypes.POINTER(ctypes.c_double)
    ip = ctypes.POINTER(ctypes.c_int)
    i64 = ctypes.c_int64
    sig = {
        "qsf_grid_create": [ctypes.POINTER(GridDesc), vp, ctypes.POINTER(vp)],
        "qsf_grid_destroy": [vp],
        "qsf_grid_size": [vp, ctypes.POINTER(i64)],
        "qsf_psi_device_ptr": [vp, ctypes.POINTER(vp)],
        "qsf_upload": [vp, dp, i64],
        "qsf_download": [vp, dp, i64],
        "qsf_synchronize": [vp],
        "qsf_fourier": [vp, ctypes.c_int],
        "qsf_evolve": [vp, ctypes.c_int, ctypes.c_int, ctypes.c_double, dp],
        "qsf_average": [vp, ctypes.c_int, ctypes.c_int, dp],
        "qsf_normalize": [vp, dp],
        "qsf_flux": [vp, dp, ctypes.c_int, ip, i64, dp],
        "qsf_mask_region": [vp, ip],
        "qsf_region_transfer": [vp, vp, ctypes.c_int, ctypes.c_int],
        "qsf_average_log": [vp, ctypes.c_int, ctypes.c_int, ctypes.c_int64],
        "qsf_read_log": [vp, dp, ctypes.c_int64],
        "qsf_add_gaussian": [vp, ctypes.c_double, ctypes.c_double],
        "qsf_step": [vp, ctypes.POINTER(StepDesc), dp, ctypes.POINTER(i64)],
        "qsf_fft_plan_radices": [i64, ip, ip],
        "qsf_batch_create": [vp, ctypes.POINTER(vp)],
        "qsf_batch_destroy": [vp],
        "qsf_batch_add": [vp, vp, ctypes.POINTER(StepDesc), ctypes.POINTER(i64)],
        "qsf_batch_remove": [vp, i64],
        "qsf_batch_run": [vp, i64, ctypes.POINTER(i64)],
        "qsf_batch_result": [vp, i64, dp, ctypes.POINTER(i64)],
        "qsf_server_start": [ctypes.POINTER(ServerConfig), ctypes.POINTER(vp)],
        "qsf_server_submit": [vp, ctypes.POINTER(Request), ctypes.POINTER(i64)],
        "qsf_server_poll": [vp, i64, ctypes.POINTER(Result), ip],
        "qsf_server_wait": [vp, i64, ctypes.c_double, ctypes.POINTER(Result)],
        "qsf_server_stats_get": [vp, ctypes.POINTER(ServerStats)],
        "qsf_server_stop": [vp],
        "qsf_server_cancel": [vp, i64],
        "qsf_save": [vp, ctypes.c_char_p, ctypes.POINTER(DumpFormat), ctypes.c_char_p, ctypes.c_char_p,
                     ctypes.c_size_t],
        "qsf_load": [vp, ctypes.c_char_p, ctypes.c_char_p, ip, dp],
        "qsf_orthogonalize_with": [vp, ctypes.c_char_p, ctypes.c_char_p, dp, dp],
        "qsf_backup": [vp, i64, ctypes.c_char_p],
        "qsf_restore": [vp, ctypes.c_char_p, ctypes.POINTER(i64)],
        "qsf_remove_backups": [ctypes.c_char_p],
        "qsf_average_der": [vp, ctypes.c_int, dp],
        "qsf_antisymmetrize": [vp, ctypes.c_int],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    L.qsf_last_error.argtypes = []
    L.qsf_last_error.restype = ctypes.c_char_p
    _lib = L
    return L


def check(rc: int, where: str) -> None:
    if rc != QSF_OK:
        raise QsfError(rc, where, lib().qsf_last_error().decode(errors="replace"))


def exported_symbols(header: str):
    """Names of the functions declared in a C header (for ABI completeness checks)."""
    import re
    text = open(header).read()
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(qsf_\w+)\s*\(", text, re.M)))

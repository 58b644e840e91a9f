"""ctypes loader of libfv3g.so (the CUDA implementation).  No fallback: if the
library cannot be built or loaded, every call raises."""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

DP = C.POINTER(C.c_double)
IP = C.POINTER(C.c_int)
VP = C.c_void_p

FV3G_FP64, FV3G_MIXED = 0, 1
FIELDS = dict(Q=0, DELP=1, CX=2, CY=3, MFX=4, MFY=5, Q_REMAPPED=6, DELP_OUT=7)
ERRORS = {-1: "FV3G_E_ARG", -2: "FV3G_E_CUDA", -3: "FV3G_E_COURANT", -4: "FV3G_E_NONFINITE", -5: "FV3G_E_DELP",
          -6: "FV3G_E_UNSUPPORTED", -7: "FV3G_E_NOMEM", -8: "FV3G_E_CHECKSUM"}

# every symbol include/fv3g.h declares (checked by the test-suite)
EXPORTS = (
    "fv3g_version", "fv3g_last_error", "fv3g_device_info", "fv3g_fv_tp_2d", "fv3g_tracer_2d", "fv3g_map_scalar",
    "fv3g_map1_ppm", "fv3g_map_scalar_3d", "fv3g_state_create", "fv3g_state_destroy", "fv3g_state_set_grid",
    "fv3g_state_set_levels", "fv3g_upload", "fv3g_download", "fv3g_upload_device", "fv3g_download_device",
    "fv3g_tracer_2d_batched", "fv3g_remap_batched", "fv3g_step", "fv3g_mass_sum", "fv3g_state_error",
    "fv3g_field_info", "fv3g_upload_async", "fv3g_download_async", "fv3g_stream_sync", "fv3g_set_timing",
    "fv3g_kernel_times", "fv3g_remap_columns_noalloc", "fv3g_fv_tp_2d_tl", "fv3g_fv_tp_2d_ad", "fv3g_map1_ppm_tl",
    "fv3g_map1_ppm_ad", "fv3g_state_autotune", "fv3g_state_widths", "fv3g_step_host", "fv3g_tracer_2d_1L", "fv3g_ensemble_create",
    "fv3g_ensemble_step", "fv3g_ensemble_destroy", "fv3g_fillz", "fv3g_pressure_vars", "fv3g_fillz_batched",
    "fv3g_tracer_2d_nested", "fv3g_nc_open", "fv3g_nc_close", "fv3g_nc_nvars", "fv3g_nc_var_info", "fv3g_nc_checksum",
    "fv3g_nc_read", "fv3g_state_read_restart", "fv3g_state_write_restart", "fv3g_state_nsplt",
    "fv3g_state_set_tracer_pairs", "fv3g_state_tracer_pairs", "fv3g_state_set_mass_fix", "fv3g_state_step_tl", "fv3g_state_step_ad", "fv3g_map1_q2", "fv3g_state_remap_fields",
    "fv3g_state_set_remap_form", "fv3g_state_remap_form",
)


class Fv3gError(RuntimeError):
    def __init__(self, code: int, fn: str, msg: str):
        super().__init__(f"{fn} failed with {ERRORS.get(code, code)}: {msg}")
        self.code = code


class Bounds(C.Structure):
    _fields_ = [(k, C.c_int) for k in ("is_", "ie", "js", "je", "isd", "ied", "jsd", "jed", "ng")]


class Grid(C.Structure):
    _fields_ = [("dx", DP), ("dy", DP), ("dxa", DP), ("dya", DP), ("area", DP), ("rarea", DP), ("sin_sg", DP),
                ("sw_corner", C.c_int), ("se_corner", C.c_int), ("nw_corner", C.c_int), ("ne_corner", C.c_int),
                ("nested", C.c_int), ("del6_u", DP), ("del6_v", DP), ("da_min", C.c_double)]


class StateDesc(C.Structure):
    _fields_ = [("n", C.c_int), ("ntiles", C.c_int), ("npz", C.c_int), ("nq", C.c_int), ("precision", C.c_int),
                ("hord", C.c_int), ("kord", C.c_int), ("iv", C.c_int), ("q_min", C.c_double),
                ("warps_per_cta", C.c_int), ("nord_tr", C.c_int), ("trdm", C.c_double), ("lim_fac", C.c_double),
                ("fill", C.c_int), ("edge_sync", C.c_int), ("mass_fix", C.c_int),
                ("independent_tiles", C.c_int)]


class NestBC(C.Structure):
    _fields_ = [(k, DP) for k in ("west_t0", "west_t1", "east_t0", "east_t1", "south_t0", "south_t1", "north_t0",
                                  "north_t1")]


HALO_FN = C.CFUNCTYPE(None, DP, C.c_int, C.c_int, VP)

_lib = None


def load(build_if_needed: bool = True):
    """Load (building first if needed) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.build() if build_if_needed else _build.LIB
    if not os.path.exists(path):
        raise RuntimeError(f"fv3g CUDA library missing at {path}")
    L = C.CDLL(path)
    for name in EXPORTS:
        getattr(L, name).restype = C.c_int
    L.fv3g_last_error.argtypes = [C.c_char_p, C.c_int]
    L.fv3g_device_info.argtypes = [C.c_char_p, C.c_int]
    _lib = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(512)
    load().fv3g_last_error(buf, 512)
    return buf.value.decode(errors="replace")


def check(rc: int, fn: str) -> int:
    if rc != 0:
        raise Fv3gError(rc, fn, last_error())
    return rc


def call(name: str, *args) -> int:
    return check(getattr(load(), name)(*args), name)

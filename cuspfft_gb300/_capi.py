"""ctypes binding of the C ABI declared in include/gbspfft.h.

The shared library is built in-tree (cuspfft_gb300/_build/libgbspfft.so) by
cuspfft_gb300.build; importing this module loads it and fails loudly when it
is missing: there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

_PKG = Path(__file__).resolve().parent
LIB_PATH = _PKG / "_build" / "libgbspfft.so"

GBSP_OK = 0
GBSP_ERR_INVALID = 1
GBSP_ERR_CUDA = 2
GBSP_ERR_ALLOC = 3
GBSP_ERR_UNSUPPORTED = 4
GBSP_ERR_IO = 5
GBSP_ERR_NOT_BUILT = 6
GBSP_LEN_POW2 = 2
GBSP_LEN_3SMOOTH = 3
GBSP_LEN_7SMOOTH = 7
GBSP_PLANNER_MODEL = 0
GBSP_PLANNER_LEARNED = 1
GBSP_STREAM_TILE_AUTO = -1  # GbspOptions.stream_tile_rows: slabs for the automatic tile
GBSP_N_PASS1_SHAPES = 8
GBSP_N_FEATURES = 36
GBSP_MLP_HIDDEN = 64

# Every symbol include/gbspfft.h declares; tests check the library exports them.
EXPORTED = (
    "gbsp_version", "gbsp_status_string", "gbsp_last_error", "gbsp_read_mtx", "gbsp_free",
    "gbsp_build_compact_csc", "gbsp_next_smooth", "gbsp_plan_create", "gbsp_plan_get_info",
    "gbsp_plan_destroy", "gbsp_execute", "gbsp_execute_profiled", "gbsp_column_sums",
    "gbsp_plan_error_flags", "gbsp_device_flags_status", "gbsp_execute_noalloc", "gbsp_batch_create", "gbsp_batch_set_outputs",
    "gbsp_batch_execute", "gbsp_batch_graph_launch", "gbsp_batch_plan_info", "gbsp_batch_error_flags",
    "gbsp_batch_destroy", "gbsp_plan_candidates", "gbsp_plan_features", "gbsp_autotune", "gbsp_mlp_param_count",
    "gbsp_mlp_forward", "gbsp_mlp_work_floats", "gbsp_mlp_backward", "gbsp_mlp_adam", "gbsp_cost_model_set", "gbsp_cost_model_set_domain",
    "gbsp_execute_to_host", "gbsp_set_memory_cache",
)


class GbspOptions(C.Structure):
    _fields_ = [
        ("length_policy", C.c_int),
        ("u_tile", C.c_int),
        ("kahan_min_degree", C.c_int),
        ("index_bytes", C.c_int),
        ("max_channel_len", C.c_int),
        ("rows_threads", C.c_int),
        ("row_table_mode", C.c_int),
        ("radix", C.c_int * 8),
        ("pass1_shape", C.c_int),
        ("planner", C.c_int),
        ("channel_mode", C.c_int),
        ("stream_tile_rows", C.c_int),
        ("exact_phases", C.c_int),
        ("force_bluestein", C.c_int),
    ]

    def radices(self) -> tuple:
        return tuple(r for r in self.radix if r > 0)


class GbspPlanInfo(C.Structure):
    _fields_ = [
        ("rows", C.c_int), ("cols", C.c_int), ("nnz", C.c_int), ("n_active", C.c_int),
        ("fft_len", C.c_int), ("channels", C.c_int), ("channel_len", C.c_int),
        ("n_stages", C.c_int), ("radix", C.c_int * 16), ("output_cols", C.c_int),
        ("output_pitch", C.c_int), ("half_rows", C.c_int), ("u_tile", C.c_int),
        ("index_bytes", C.c_int), ("row_table_mode", C.c_int), ("rows_threads", C.c_int),
        ("device_bytes", C.c_size_t), ("pass1_shape", C.c_int), ("planner", C.c_int), ("channel_mode", C.c_int),
        ("exact_phases", C.c_int), ("direct", C.c_int),
    ]

    def as_dict(self) -> dict:
        d = {name: getattr(self, name) for name, _ in self._fields_ if name != "radix"}
        d["radix"] = [self.radix[i] for i in range(self.n_stages)]
        return d


class GbspMatrix(C.Structure):
    _fields_ = [
        ("rows", C.c_int), ("cols", C.c_int), ("n_active", C.c_int), ("nnz", C.c_int),
        ("col_ptr", C.POINTER(C.c_int)), ("row_idx", C.POINTER(C.c_int)),
        ("sparse_cols", C.POINTER(C.c_int)),
    ]


class GbspTuneEntry(C.Structure):
    _fields_ = [("opts", GbspOptions), ("ms_pass1", C.c_float), ("ms_rows", C.c_float)]


class GbspError(RuntimeError):
    def __init__(self, status: int, what: str, msg: str):
        super().__init__(f"{what}: {status_string(status)}: {msg}")
        self.status = status


_lib = None


def load(build_if_missing: bool = True) -> C.CDLL:
    """Returns the loaded library, building it first if it is absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists() and build_if_missing and os.environ.get("GBSP_NO_AUTOBUILD") != "1":
        from . import build as _build
        _build.build()
    if not LIB_PATH.exists():
        raise RuntimeError(f"cuspfft_gb300 native library missing: {LIB_PATH} (run cuspfft_gb300.build)")
    lib = C.CDLL(str(LIB_PATH))
    vp, ip, i32 = C.c_void_p, C.POINTER(C.c_int), C.c_int
    lib.gbsp_version.restype = i32
    lib.gbsp_status_string.restype = C.c_char_p
    lib.gbsp_status_string.argtypes = [i32]
    lib.gbsp_last_error.argtypes = [C.c_char_p, C.c_size_t]
    lib.gbsp_read_mtx.argtypes = [C.c_char_p, ip, ip, ip, C.POINTER(ip), C.POINTER(ip)]
    lib.gbsp_free.argtypes = [vp]
    lib.gbsp_free.restype = None
    lib.gbsp_build_compact_csc.argtypes = [i32, i32, i32, ip, ip, ip, ip, ip, ip]
    lib.gbsp_next_smooth.argtypes = [i32, i32]
    lib.gbsp_plan_create.argtypes = [i32, i32, i32, i32, ip, ip, ip, C.POINTER(GbspOptions), vp,
                                     C.POINTER(vp)]
    lib.gbsp_plan_get_info.argtypes = [vp, C.POINTER(GbspPlanInfo)]
    lib.gbsp_plan_destroy.argtypes = [vp]
    lib.gbsp_set_memory_cache.argtypes = [C.c_size_t]
    lib.gbsp_execute.argtypes = [vp, vp, C.c_size_t, vp]
    lib.gbsp_execute_profiled.argtypes = [vp, vp, C.c_size_t, vp, C.POINTER(C.c_float),
                                           C.POINTER(C.c_float)]
    lib.gbsp_column_sums.argtypes = [vp, i32, i32, vp, C.c_size_t, vp]
    lib.gbsp_plan_error_flags.argtypes = [vp, ip]
    lib.gbsp_device_flags_status.argtypes = [i32]
    lib.gbsp_execute_noalloc.argtypes = [vp, vp, C.c_size_t, vp]
    lib.gbsp_batch_create.argtypes = [i32, C.POINTER(GbspMatrix), C.POINTER(GbspOptions), vp, C.POINTER(vp)]
    lib.gbsp_batch_set_outputs.argtypes = [vp, C.POINTER(vp), C.POINTER(C.c_size_t)]
    lib.gbsp_batch_execute.argtypes = [vp, vp]
    lib.gbsp_batch_graph_launch.argtypes = [vp, vp]
    lib.gbsp_batch_plan_info.argtypes = [vp, i32, C.POINTER(GbspPlanInfo)]
    lib.gbsp_batch_error_flags.argtypes = [vp, ip]
    lib.gbsp_batch_destroy.argtypes = [vp]
    op = C.POINTER(GbspOptions)
    fp = C.POINTER(C.c_float)
    lib.gbsp_plan_candidates.argtypes = [i32, i32, op, i32, op, i32, ip, ip]
    lib.gbsp_plan_features.argtypes = [i32, i32, i32, i32, ip, op, fp]
    lib.gbsp_autotune.argtypes = [i32, i32, i32, i32, ip, ip, ip, op, i32, i32, vp, op, C.POINTER(GbspTuneEntry),
                                  i32, ip, ip]
    lib.gbsp_mlp_param_count.argtypes = [i32]
    lib.gbsp_mlp_param_count.restype = C.c_size_t
    lib.gbsp_mlp_work_floats.argtypes = [i32]
    lib.gbsp_mlp_work_floats.restype = C.c_size_t
    lib.gbsp_mlp_forward.argtypes = [vp, i32, vp, i32, vp, vp]
    lib.gbsp_mlp_backward.argtypes = [vp, i32, vp, vp, i32, vp, vp, vp, vp]
    lib.gbsp_mlp_adam.argtypes = [vp, vp, vp, vp, C.c_size_t, C.c_float, C.c_float, C.c_float, C.c_float, i32, vp]
    lib.gbsp_cost_model_set.argtypes = [fp, i32, fp, fp]
    lib.gbsp_cost_model_set_domain.argtypes = [i32, fp, fp]
    lib.gbsp_execute_to_host.argtypes = [vp, vp, C.c_size_t, i32, vp]
    for name in EXPORTED:
        if name not in ("gbsp_status_string", "gbsp_free", "gbsp_mlp_param_count", "gbsp_mlp_work_floats"):
            getattr(lib, name).restype = i32
    _lib = lib
    return lib


def status_string(status: int) -> str:
    return load().gbsp_status_string(status).decode()


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    load().gbsp_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(status: int, what: str) -> None:
    if status != GBSP_OK:
        raise GbspError(status, what, last_error())

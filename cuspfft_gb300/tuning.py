"""Autotuner front end: tuning candidates, cost-model features and exhaustive
measurement (gbsp_plan_candidates / gbsp_plan_features / gbsp_autotune in
include/gbspfft.h).

The reference fixes its configuration (--csc-tile and the 9/3/2 radix
order, src/sparse_fft_bluestein.cu:1996-2011); here every matrix has a set
of candidates -- the analytic model's cheapest (radix sequence, row block)
choices crossed with the pass-1 shapes that fit -- and the tuner measures
them all.  The spectrum does not depend on the choice.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from ._capi import GBSP_N_FEATURES, GbspOptions, GbspTuneEntry, check, load
from .sparse_fft import COOMatrix, CompactCSC, _ip, _stream_handle, make_compact_csc, make_options

# feature slices: matrix, row choice, pass-1 shape
F_MATRIX = slice(0, 18)
F_ROWS = slice(18, 28)
F_PASS1 = slice(28, 36)
MAX_CANDIDATES = 8 * 8  # row choices x pass-1 shapes (GBSP_N_PASS1_SHAPES)


def candidates(rows: int, cols: int, base: Optional[GbspOptions] = None, max_rows_cands: int = 8,
               **fields) -> tuple[list[GbspOptions], int, int]:
    """(candidates, n_rows, n_p1); candidate i * n_p1 + j pairs row choice i
    with pass-1 shape j."""
    lib = load()
    o = make_options(base, **fields)
    out = (GbspOptions * MAX_CANDIDATES)()
    nr, npp = C.c_int(), C.c_int()
    check(lib.gbsp_plan_candidates(rows, cols, C.byref(o), max_rows_cands, out, MAX_CANDIDATES, C.byref(nr),
                                   C.byref(npp)), "gbsp_plan_candidates")
    return [out[i] for i in range(nr.value * npp.value)], nr.value, npp.value


def features(coo: COOMatrix, cand: GbspOptions, csc: Optional[CompactCSC] = None) -> np.ndarray:
    lib = load()
    csc = csc if csc is not None else make_compact_csc(coo)
    cp = np.ascontiguousarray(csc.col_ptr, np.int32)
    f = np.zeros(GBSP_N_FEATURES, np.float32)
    check(lib.gbsp_plan_features(coo.rows, coo.cols, csc.n_sparse_cols, coo.nnz, _ip(cp), C.byref(cand),
                                 f.ctypes.data_as(C.POINTER(C.c_float))), "gbsp_plan_features")
    return f


@dataclass
class TuneResult:
    best: GbspOptions
    candidates: list            # GbspOptions, i * n_p1 + j
    n_rows: int
    n_p1: int
    ms_rows: np.ndarray         # [n_rows]: Bluestein rows under row choice i
    ms_pass1: np.ndarray        # [n_p1]: pass 1 under shape j

    def total(self) -> np.ndarray:
        """[n_rows, n_p1] composed device time of every candidate."""
        return self.ms_rows[:, None] + self.ms_pass1[None, :]


def autotune(coo: COOMatrix, *, max_rows_cands: int = 8, reps: int = 3, stream=None,
             csc: Optional[CompactCSC] = None, base: Optional[GbspOptions] = None, **fields) -> TuneResult:
    """Measures every candidate of the matrix on the current GPU."""
    lib = load()
    csc = csc if csc is not None else make_compact_csc(coo)
    o = make_options(base, **fields)
    cp = np.ascontiguousarray(csc.col_ptr, np.int32)
    ri = np.ascontiguousarray(csc.row_idx if coo.nnz else np.zeros(1, np.int32), np.int32)
    sc = np.ascontiguousarray(csc.sparse_cols if csc.n_sparse_cols else np.zeros(1, np.int32), np.int32)
    best = GbspOptions()
    ent = (GbspTuneEntry * MAX_CANDIDATES)()
    nr, npp = C.c_int(), C.c_int()
    check(lib.gbsp_autotune(coo.rows, coo.cols, csc.n_sparse_cols, coo.nnz, _ip(cp), _ip(ri), _ip(sc), C.byref(o),
                            max_rows_cands, reps, _stream_handle(stream), C.byref(best), ent, MAX_CANDIDATES,
                            C.byref(nr), C.byref(npp)), "gbsp_autotune")
    n_r, n_p = nr.value, npp.value
    cands = [ent[i].opts for i in range(n_r * n_p)]
    ms_rows = np.array([ent[i * n_p].ms_rows for i in range(n_r)], np.float64)
    ms_p1 = np.array([ent[j].ms_pass1 for j in range(n_p)], np.float64)
    return TuneResult(best, cands, n_r, n_p, ms_rows, ms_p1)

#!/usr/bin/env python3
"""Generates the golden fixtures in tests/golden/ from the reference's own
host code (oracle/_ref/libref_host.so, compiled from the reference sources by
oracle/build_ref.sh).  Run here, where the reference tree exists; the
fixtures travel with the repository so the tests need no reference at run
time.

  mtx/*.mtx            small Matrix Market inputs written by this script
                       (general, pattern, symmetric, skew-symmetric,
                       duplicates, comments, blank lines, empty, malformed)
  reader_csc.npz       per input: read_mtx's COO and make_compact_csc's CSC,
                       or the reference's error message
  tables.npz           make_bluestein_chirp / make_bluestein_b tables,
                       next_3_smooth / next_7_smooth / factor_3_smooth values
  spectra.npz          FP64 spectra of tiny matrices (from oracle/fp64.py, an
                       independent definition) for regression checks

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT))

from oracle import fp64, refhost  # noqa: E402

MTX = {
    "general_real": "%%MatrixMarket matrix coordinate real general\n% a comment\n4 5 6\n1 2 0.5\n3 1 -2\n4 5 1e-3\n2 2 7\n1 2 9\n4 1 3\n",
    "pattern": "%%MatrixMarket matrix coordinate pattern general\n3 3 4\n1 1\n2 3\n3 2\n1 3\n",
    "symmetric": "%%MatrixMarket matrix coordinate real symmetric\n%\n%\n5 5 5\n1 1 1\n2 1 1\n4 2 1\n5 5 2\n5 3 4\n",
    "skew_symmetric": "%%MatrixMarket matrix coordinate real skew-symmetric\n4 4 3\n2 1 1\n3 1 -1\n4 3 2\n",
    "Symmetric_caps": "%%MatrixMarket matrix coordinate integer Symmetric\n3 3 2\n2 1 5\n3 3 1\n",
    "duplicates": "%%MatrixMarket matrix coordinate real general\n3 4 6\n1 1 1\n1 1 2\n2 4 1\n2 4 1\n3 2 0\n1 1 3\n",
    "blank_before_dims": "%%MatrixMarket matrix coordinate real general\n\n% c\n\n2 3 2\n1 3 1\n2 1 1\n",
    "one_by_one": "%%MatrixMarket matrix coordinate real general\n1 1 1\n1 1 5\n",
    "empty": "%%MatrixMarket matrix coordinate real general\n6 7 0\n",
    "wide": "%%MatrixMarket matrix coordinate pattern general\n2 40 5\n1 40\n2 39\n1 1\n2 20\n1 20\n",
    "tall_unsorted": "%%MatrixMarket matrix coordinate pattern general\n9 2 7\n9 2\n1 1\n5 2\n5 1\n2 2\n9 1\n3 2\n",
    # malformed inputs: the reference throws; the message is the fixture
    "bad_header": "%%NotMatrixMarket matrix coordinate real general\n2 2 1\n1 1 1\n",
    "bad_dims": "%%MatrixMarket matrix coordinate real general\n2 x 1\n1 1 1\n",
    "truncated": "%%MatrixMarket matrix coordinate real general\n3 3 3\n1 1 1\n2 2 1\n",
    "bad_entry": "%%MatrixMarket matrix coordinate real general\n3 3 2\n1 1 1\nfoo 2 1\n",
    "only_comments": "%%MatrixMarket matrix coordinate real general\n% nothing else\n",
}

CHIRP_N = [1, 2, 3, 5, 7, 16, 64, 100, 257, 1000, 2048, 3001]
B_NL = [(1, 2), (2, 3), (5, 9), (7, 16), (64, 128), (100, 199), (257, 513), (1000, 2000), (2048, 4096),
        (3001, 6048)]
SMOOTH_N = list(range(1, 400)) + [4095, 4097, 6001, 16437, 33411, 80841, 123456, 200001]
FACTOR_N = [1, 2, 3, 4, 6, 8, 9, 12, 18, 27, 81, 96, 243, 729, 1024, 4096, 6144, 17496, 34992, 82944]


def main() -> None:
    if not refhost.available():
        sys.exit("oracle/_ref/libref_host.so is missing: run oracle/build_ref.sh first")
    mdir = HERE / "mtx"
    mdir.mkdir(exist_ok=True)
    reader = {}
    for name, text in MTX.items():
        path = mdir / f"{name}.mtx"
        path.write_text(text)
        try:
            rows, cols, r, c = refhost.read_mtx(str(path))
        except RuntimeError as e:
            # messages embed the path: keep only the part before it
            reader[f"{name}/error"] = np.array(str(e).split(": ")[0])
            continue
        sc, cp, ri = refhost.make_compact_csc(rows, cols, r, c)
        reader[f"{name}/dims"] = np.array([rows, cols], np.int32)
        reader[f"{name}/row_idx"] = r.astype(np.int32)
        reader[f"{name}/col_idx"] = c.astype(np.int32)
        reader[f"{name}/sparse_cols"] = sc.astype(np.int32)
        reader[f"{name}/col_ptr"] = cp.astype(np.int32)
        reader[f"{name}/csc_row_idx"] = ri.astype(np.int32)
    # CSC builder on COO inputs that are not row-sorted (stable-order check)
    g = np.random.default_rng(12)
    for k in range(4):
        rows, cols, n = int(g.integers(1, 60)), int(g.integers(1, 60)), int(g.integers(0, 300))
        r = g.integers(0, rows, n).astype(np.int32)
        c = g.integers(0, cols, n).astype(np.int32)
        sc, cp, ri = refhost.make_compact_csc(rows, cols, r, c)
        reader[f"csc_random{k}/dims"] = np.array([rows, cols], np.int32)
        reader[f"csc_random{k}/row_idx"] = r
        reader[f"csc_random{k}/col_idx"] = c
        reader[f"csc_random{k}/sparse_cols"] = sc
        reader[f"csc_random{k}/col_ptr"] = cp
        reader[f"csc_random{k}/csc_row_idx"] = ri
    np.savez_compressed(HERE / "reader_csc.npz", **reader)

    tables = {}
    for n in CHIRP_N:
        tables[f"chirp/{n}"] = refhost.bluestein_chirp(n)
    for n, L in B_NL:
        tables[f"b/{n}/{L}"] = refhost.bluestein_b(n, L)
    tables["smooth/n"] = np.array(SMOOTH_N, np.int64)
    tables["smooth/3"] = np.array([refhost.next_3_smooth(n) for n in SMOOTH_N], np.int64)
    tables["smooth/7"] = np.array([refhost.next_7_smooth(n) for n in SMOOTH_N], np.int64)
    for n in FACTOR_N:
        tables[f"factor3/{n}"] = np.array(refhost.factor_3_smooth(n), np.int32)
    np.savez_compressed(HERE / "tables.npz", **tables)

    spectra = {}
    for k, (rows, cols, n) in enumerate([(5, 7, 9), (8, 8, 20), (11, 4, 15), (3, 13, 10), (16, 9, 40)]):
        r = g.integers(0, rows, n)
        c = g.integers(0, cols, n)
        key = np.unique(r * cols + c)
        r, c = (key // cols).astype(np.int32), (key % cols).astype(np.int32)
        spectra[f"m{k}/dims"] = np.array([rows, cols], np.int32)
        spectra[f"m{k}/row_idx"] = r
        spectra[f"m{k}/col_idx"] = c
        spectra[f"m{k}/F"] = fp64.direct_dft_fp64(rows, cols, r, c)
    np.savez_compressed(HERE / "spectra.npz", **spectra)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()

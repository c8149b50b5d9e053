"""The oracle's and the library's host path against golden fixtures generated
from the reference's own code (tests/golden/make_golden.py).  Bit-exact: these
are integer / byte results and FP64->FP32 tables."""
from pathlib import Path

import numpy as np
import pytest

import cuspfft_gb300 as gb
from oracle import fp64, ref_port

G = Path(__file__).resolve().parent / "golden"
READER = np.load(G / "reader_csc.npz")
TABLES = np.load(G / "tables.npz")
SPECTRA = np.load(G / "spectra.npz")
NAMES = sorted({k.split("/")[0] for k in READER.files if not k.startswith("csc_random")})
CSC_CASES = sorted({k.split("/")[0] for k in READER.files if "/sparse_cols" in k})


@pytest.mark.parametrize("name", NAMES)
def test_reader_library_and_oracle(name):
    path = str(G / "mtx" / f"{name}.mtx")
    if f"{name}/error" in READER.files:
        msg = str(READER[f"{name}/error"])
        with pytest.raises(RuntimeError, match=msg):
            gb.read_mtx(path)
        with pytest.raises(RuntimeError, match=msg):
            ref_port.read_mtx(path)
        return
    rows, cols = READER[f"{name}/dims"].tolist()
    coo = gb.read_mtx(path)
    assert (coo.rows, coo.cols) == (rows, cols)
    assert np.array_equal(coo.row_idx, READER[f"{name}/row_idx"])
    assert np.array_equal(coo.col_idx, READER[f"{name}/col_idx"])
    r2, c2, ri, ci = ref_port.read_mtx(path)
    assert (r2, c2) == (rows, cols)
    assert np.array_equal(ri, READER[f"{name}/row_idx"]) and np.array_equal(ci, READER[f"{name}/col_idx"])


@pytest.mark.parametrize("name", CSC_CASES)
def test_compact_csc_library_and_oracle(name):
    rows, cols = READER[f"{name}/dims"].tolist()
    r, c = READER[f"{name}/row_idx"], READER[f"{name}/col_idx"]
    csc = gb.make_compact_csc(gb.COOMatrix(rows, cols, r, c))
    assert np.array_equal(csc.sparse_cols, READER[f"{name}/sparse_cols"])
    assert np.array_equal(csc.col_ptr, READER[f"{name}/col_ptr"])
    assert np.array_equal(csc.row_idx, READER[f"{name}/csc_row_idx"])
    sc, cp, ri = ref_port.make_compact_csc(rows, cols, r, c)
    assert np.array_equal(sc, READER[f"{name}/sparse_cols"])
    assert np.array_equal(cp, READER[f"{name}/col_ptr"])
    assert np.array_equal(ri, READER[f"{name}/csc_row_idx"])


def test_smooth_lengths():
    ns = TABLES["smooth/n"]
    for n, s3, s7 in zip(ns, TABLES["smooth/3"], TABLES["smooth/7"]):
        assert gb.next_smooth(int(n), gb.GBSP_LEN_3SMOOTH) == s3
        assert gb.next_smooth(int(n), gb.GBSP_LEN_7SMOOTH) == s7
        assert ref_port.next_smooth(int(n), False) == s3
        assert ref_port.next_smooth(int(n), True) == s7


def test_power_of_two_lengths():
    # the reference's pow2 methods: fft_len = next_power_of_two(2*cols - 1)
    assert gb.next_smooth(2 * 8219 - 1, gb.GBSP_LEN_POW2) == 32768
    for n in list(range(1, 5000)) + [65535, 65536, 65537, 80841, (1 << 27) + 1]:
        assert gb.next_smooth(n, gb.GBSP_LEN_POW2) == ref_port.next_power_of_two(n)


def test_factor_3_smooth():
    for k in TABLES.files:
        if k.startswith("factor3/"):
            n = int(k.split("/")[1])
            assert ref_port.factor_3_smooth(n) == TABLES[k].tolist()


def test_bluestein_tables_bit_exact():
    for k in TABLES.files:
        if k.startswith("chirp/"):
            n = int(k.split("/")[1])
            assert np.array_equal(ref_port.bluestein_chirp(n).view(np.uint32), TABLES[k].view(np.uint32))
        if k.startswith("b/"):
            _, n, L = k.split("/")
            assert np.array_equal(ref_port.bluestein_b(int(n), int(L)).view(np.uint32), TABLES[k].view(np.uint32))


def test_fp64_oracle_on_golden_spectra():
    for k in SPECTRA.files:
        if k.endswith("/F"):
            m = k.split("/")[0]
            rows, cols = SPECTRA[f"{m}/dims"].tolist()
            r, c = SPECTRA[f"{m}/row_idx"], SPECTRA[f"{m}/col_idx"]
            F = fp64.spectrum_rows_fp64(rows, cols, r, c)
            assert np.max(np.abs(F - SPECTRA[k])) < 1e-10


def test_live_reference_host_code():
    """Randomised comparison with the reference's compiled host functions,
    where the reference tree (and so oracle/_ref) is present."""
    from oracle import refhost
    if not refhost.available():
        pytest.skip("reference host library not built here")
    g = np.random.default_rng(3)
    for _ in range(20):
        rows, cols, n = int(g.integers(1, 300)), int(g.integers(1, 300)), int(g.integers(0, 2000))
        r = g.integers(0, rows, n).astype(np.int32)
        c = g.integers(0, cols, n).astype(np.int32)
        sc, cp, ri = refhost.make_compact_csc(rows, cols, r, c)
        csc = gb.make_compact_csc(gb.COOMatrix(rows, cols, r, c))
        assert np.array_equal(csc.sparse_cols, sc) and np.array_equal(csc.col_ptr, cp)
        assert np.array_equal(csc.row_idx, ri)
    for n in g.integers(1, 100000, 50):
        assert gb.next_smooth(int(n), 3) == refhost.next_3_smooth(int(n))
        assert gb.next_smooth(int(n), 7) == refhost.next_7_smooth(int(n))
        assert gb.next_smooth(int(n), gb.GBSP_LEN_POW2) == refhost.next_power_of_two(int(n))

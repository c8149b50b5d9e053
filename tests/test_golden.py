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


def test_live_reference_reader_fuzz(tmp_path):
    """Random Matrix Market files read by this library and by the reference's
    compiled read_mtx (where the reference tree is present): the same COO,
    and through make_compact_csc the same CSC, bit for bit.  Header kinds,
    comment lines, explicit values (zeros included), duplicates and diagonal
    entries vary; every entry is in range (the reference does not check)."""
    from oracle import refhost
    if not refhost.available():
        pytest.skip("reference host library not built here")
    g = np.random.default_rng(11)
    kinds = [("pattern", "general"), ("real", "general"), ("integer", "general"), ("pattern", "symmetric"),
             ("real", "symmetric"), ("real", "skew-symmetric")]
    for t in range(60):
        field, sym = kinds[t % len(kinds)]
        rows = int(g.integers(1, 200))
        cols = rows if sym != "general" else int(g.integers(1, 200))
        n = int(g.integers(0, 600))
        r = g.integers(1, rows + 1, n)
        c = g.integers(1, cols + 1, n)
        if sym != "general":  # lower triangle, as symmetric files store it
            r, c = np.maximum(r, c), np.minimum(r, c)
        if n and g.random() < 0.5:  # duplicates
            k = int(g.integers(1, n + 1))
            r, c = np.concatenate([r, r[:k]]), np.concatenate([c, c[:k]])
        lines = [f"%%MatrixMarket matrix coordinate {field} {sym}"]
        lines += [f"% comment {i}" for i in range(int(g.integers(0, 3)))]
        lines.append(f"{rows} {cols} {r.size}")
        for rr, cc in zip(r, c):
            if field == "pattern":
                lines.append(f"{rr} {cc}")
            elif field == "integer":
                lines.append(f"{rr} {cc} {int(g.integers(-3, 4))}")
            else:
                lines.append(f"{rr} {cc} {float(g.choice([0.0, 1.5, -2.25, 1e-300]))}")
        path = tmp_path / f"f{t}.mtx"
        path.write_text("\n".join(lines) + "\n")
        want = refhost.read_mtx(str(path))
        coo = gb.read_mtx(str(path))
        assert (coo.rows, coo.cols) == want[:2], path.read_text()[:200]
        assert np.array_equal(coo.row_idx, want[2]) and np.array_equal(coo.col_idx, want[3]), f"file {t}"
        sc, cp, ri = refhost.make_compact_csc(coo.rows, coo.cols, want[2], want[3])
        csc = gb.make_compact_csc(coo)
        assert np.array_equal(csc.sparse_cols, sc) and np.array_equal(csc.col_ptr, cp)
        assert np.array_equal(csc.row_idx, ri)


def test_live_reference_bluestein_tables_random_lengths():
    """The oracle's restatement of the reference's chirp and b tables equals
    the compiled reference functions bit for bit on random lengths (where the
    reference tree is present), beyond the golden ones."""
    from oracle import refhost
    if not refhost.available():
        pytest.skip("reference host library not built here")
    g = np.random.default_rng(2)
    for n in [int(v) for v in g.integers(2, 60000, 30)] + [8219, 16706, 40421, 65535]:
        for seven in (False, True):
            L = ref_port.next_smooth(2 * n - 1, seven=seven)
            assert np.array_equal(ref_port.bluestein_chirp(n).view(np.uint32),
                                  refhost.bluestein_chirp(n).view(np.uint32)), n
            assert np.array_equal(ref_port.bluestein_b(n, L).view(np.uint32),
                                  refhost.bluestein_b(n, L).view(np.uint32)), (n, L)


def test_live_reference_factor_and_u16_rule_random():
    """factor_3_smooth on random 3-smooth lengths and the u16 packing rule on
    random sizes: the oracle restatement equals the compiled reference."""
    from oracle import refhost
    if not refhost.available():
        pytest.skip("reference host library not built here")
    g = np.random.default_rng(4)
    for n in g.integers(1, 200000, 100):
        m = ref_port.next_smooth(int(n), seven=False)
        assert refhost.factor_3_smooth(m) == list(ref_port.factor_3_smooth(m)), m
    for _ in range(100):
        r, c = int(g.integers(1, 140000)), int(g.integers(1, 140000))
        assert refhost.can_pack_u16(r, c) == ref_port.can_pack_u16(r, c), (r, c)

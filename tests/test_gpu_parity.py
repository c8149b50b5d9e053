"""Parity of the CUDA path (through the C ABI) with the FP64 oracle.

Tolerance: relative L2 error <= 1e-5 over the whole half-spectrum, the bar
the FP32 form must meet against a double-precision DFT of the same binary
matrix.  Padding columns [cols/2+1, pitch) must be exactly zero.
"""
import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import synthetic
from oracle import fp64

pytestmark = pytest.mark.gpu

REL_L2_TOL = 1e-5


def run_plan(coo, **kw):
    import torch
    with gb.Plan(coo, **kw) as plan:
        out = plan.empty_output()
        out.fill_(complex(7.0, 7.0))  # poison: every element must be overwritten
        plan.execute(out)
        torch.cuda.synchronize()
        return out.cpu().numpy(), plan.info


def check_against_oracle(coo, got, us=None, tol=REL_L2_TOL):
    fc = coo.cols // 2 + 1
    if us is None:
        ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
        sub = got[:, :fc]
    else:
        ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx, us)
        sub = got[us, :fc]
    err = fp64.rel_l2(sub, ref)
    assert err <= tol, f"rel-L2 {err:.3e} > {tol:.0e}"
    assert np.all(got[:, fc:] == 0), "padding columns must be zero"
    return err


SHAPES = [(1, 1), (1, 7), (7, 1), (2, 2), (3, 5), (17, 31), (64, 64), (101, 97), (128, 250),
          (255, 256), (300, 1001), (997, 13), (513, 2048)]


@pytest.mark.parametrize("rows,cols", SHAPES)
@pytest.mark.parametrize("policy", [gb.GBSP_LEN_3SMOOTH, gb.GBSP_LEN_7SMOOTH, gb.GBSP_LEN_POW2])
def test_random_shapes(cuda, rows, cols, policy):
    g = np.random.default_rng(rows * 1000 + cols)
    n = max(1, int(0.05 * rows * cols))
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, n), g.integers(0, cols, n))
    got, info = run_plan(coo, length_policy=policy)
    check_against_oracle(coo, got)


# cols = 333: 3-smooth L = 729 = 3^6, 7-smooth L = 672 = 2^5 * 3 * 7
@pytest.mark.parametrize("policy,max_len,channels", [
    (gb.GBSP_LEN_3SMOOTH, 250, 3), (gb.GBSP_LEN_7SMOOTH, 250, 3), (gb.GBSP_LEN_7SMOOTH, 340, 2),
    (gb.GBSP_LEN_7SMOOTH, 170, 4), (gb.GBSP_LEN_7SMOOTH, 120, 6), (gb.GBSP_LEN_7SMOOTH, 100, 7),
    (gb.GBSP_LEN_7SMOOTH, 84, 8)])
@pytest.mark.parametrize("channel_mode", [1, 2])
def test_channel_split_clusters(cuda, policy, max_len, channels, channel_mode):
    # forces the length-L convolution into K channels, run as one
    # thread-block cluster (1) or one after another in one CTA (2)
    g = np.random.default_rng(max_len)
    rows, cols = 123, 333
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, 3000), g.integers(0, cols, 3000))
    got, info = run_plan(coo, length_policy=policy, max_channel_len=max_len, channel_mode=channel_mode)
    assert info["channels"] == channels and info["channel_mode"] == channel_mode
    check_against_oracle(coo, got)


def test_channel_modes_agree_on_large_rows(cuda):
    # 16706 columns need two channels; both layouts give the same spectrum
    # to FP32 rounding
    coo = synthetic.uniform_matrix(257, 16706, 40000, seed=12)
    a, ia = run_plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, channel_mode=1)
    b, ib = run_plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, channel_mode=2)
    assert ia["channels"] == 2 and ib["channel_mode"] == 2
    assert fp64.rel_l2(a, b) < 1e-6
    check_against_oracle(coo, b, us=np.array([0, 1, 77, 128, 256]))


def test_u_tiles_and_index_width(cuda):
    coo = synthetic.uniform_matrix(257, 300, 4000, seed=9)
    base, _ = run_plan(coo)
    for kw in ({"u_tile": 1}, {"u_tile": 5}, {"u_tile": 64}, {"index_bytes": 4},
               {"kahan_min_degree": 1}, {"kahan_min_degree": -1}):
        got, _ = run_plan(coo, **kw)
        check_against_oracle(coo, got)
        assert fp64.rel_l2(got, base) < 1e-5


@pytest.mark.parametrize("index_bytes,u_tile", [(2, 0), (2, 1), (4, 0)])
@pytest.mark.parametrize("bad", [-1, 100, 1 << 20])
def test_row_index_out_of_range_is_rejected(cuda, index_bytes, u_tile, bad):
    """Row indices are range-checked on the device while they upload (u16
    narrowing staged in the scratch tile or, for a small tile, a region of its
    own); a bad one fails the plan before any transform can read it."""
    import ctypes as C
    from cuspfft_gb300 import _capi
    from cuspfft_gb300.sparse_fft import make_options
    lib = _capi.load()
    rows, cols, per_col = 100, 50, 12
    g = np.random.default_rng(5)
    ri = np.concatenate([np.sort(g.choice(rows, per_col, replace=False)) for _ in range(cols)]).astype(np.int32)
    cp = np.arange(cols + 1, dtype=np.int32) * per_col
    sc = np.arange(cols, dtype=np.int32)
    o = make_options(None, index_bytes=index_bytes, u_tile=u_tile)
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    h = C.c_void_p()
    assert lib.gbsp_plan_create(rows, cols, cols, len(ri), ip(cp), ip(ri), ip(sc), C.byref(o), None,
                                C.byref(h)) == _capi.GBSP_OK
    assert lib.gbsp_plan_destroy(h) == _capi.GBSP_OK
    ri[len(ri) // 2 + 3] = bad
    h = C.c_void_p()
    st = lib.gbsp_plan_create(rows, cols, cols, len(ri), ip(cp), ip(ri), ip(sc), C.byref(o), None, C.byref(h))
    assert st == _capi.GBSP_ERR_INVALID and not h.value
    assert "row index out of range" in _capi.last_error()


def test_half_row_table(cuda):
    # rows beyond the full-table budget use the half-circle twiddle table
    coo = synthetic.uniform_matrix(24001, 40, 20000, seed=11)
    got, info = run_plan(coo)
    assert info["row_table_mode"] == 1
    check_against_oracle(coo, got)


def test_known_answers(cuda):
    rows, cols = 12, 10
    # empty matrix -> all zeros
    empty = gb.COOMatrix(rows, cols, np.zeros(0, np.int32), np.zeros(0, np.int32))
    got, _ = run_plan(empty)
    assert np.all(got == 0)
    # one nonzero at (r0, c0): unit-modulus plane wave
    r0, c0 = 5, 3
    one = gb.COOMatrix(rows, cols, np.array([r0]), np.array([c0]))
    got, _ = run_plan(one)
    u = np.arange(rows)[:, None]
    v = np.arange(cols // 2 + 1)[None, :]
    expect = np.exp(-2j * np.pi * (u * r0 / rows + v * c0 / cols))
    assert np.max(np.abs(got[:, : cols // 2 + 1] - expect)) < 1e-5
    # a full matrix row: F[u][v] = cols * delta(v) * exp(-2 pi i u r0 / rows)
    full = gb.COOMatrix(rows, cols, np.full(cols, r0), np.arange(cols))
    got, _ = run_plan(full)
    assert abs(got[0, 0] - cols) < 1e-4
    assert np.max(np.abs(got[:, 1: cols // 2 + 1])) < 1e-4
    # F[0][0] = nnz
    coo = synthetic.uniform_matrix(50, 60, 700, seed=3)
    got, _ = run_plan(coo)
    assert abs(got[0, 0] - coo.nnz) < 1e-3 * coo.nnz


def test_symmetric_transpose_property(cuda):
    # A symmetric with rows == cols  =>  F[u][v] == F[v][u]
    coo = synthetic.uniform_powerlaw(n=301, target_nnz=3000, seed=8)
    got, _ = run_plan(coo)
    h = coo.cols // 2 + 1
    blk = got[:h, :h]
    assert fp64.rel_l2(blk, blk.T) < 1e-5


def test_column_sums(cuda):
    import torch
    coo = synthetic.uniform_matrix(211, 77, 2000, seed=5)
    with gb.Plan(coo) as plan:
        s = torch.zeros((150, 80), dtype=torch.complex64, device="cuda")
        plan.column_sums(30, 150, s)
        torch.cuda.synchronize()
        got = s.cpu().numpy()
        assert plan.error_flags() == 0
    ref = fp64.column_sums_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx, np.arange(30, 180))
    assert fp64.rel_l2(got[:, :coo.cols], ref) < 1e-6
    assert np.all(got[:, coo.cols:78] == 0)


def test_config_uniform_3001x2048_full(cuda):
    coo = synthetic.config_matrix("uniform_3001x2048")
    for policy in (gb.GBSP_LEN_3SMOOTH, gb.GBSP_LEN_7SMOOTH):
        got, info = run_plan(coo, length_policy=policy)
        check_against_oracle(coo, got)


@pytest.mark.parametrize("name", ["banded_powerlaw_8219", "uniform_powerlaw_16706"])
def test_config_sampled_rows(cuda, name):
    coo = synthetic.config_matrix(name)
    g = np.random.default_rng(0)
    us = np.unique(np.concatenate([[0, 1, coo.rows // 2, coo.rows - 1], g.integers(0, coo.rows, 12)]))
    for policy in (gb.GBSP_LEN_3SMOOTH, gb.GBSP_LEN_7SMOOTH):
        got, info = run_plan(coo, length_policy=policy)
        check_against_oracle(coo, got, us=us)


def test_reference_api_methods(cuda):
    import torch
    coo = synthetic.uniform_matrix(301, 127, 1500, seed=21)
    ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    for fn in (gb.sparse_fft_csc_bluestein_mixed_radix, gb.sparse_fft_csc_bluestein_cufft_smooth,
               gb.sparse_fft_csc_bluestein, gb.sparse_fft_csc_bluestein_smem, gb.sparse_fft_csc_bluestein_cufft,
               gb.sparse_fft_csc_stockham_binary_smem):
        res = fn(coo, 16)
        assert res.output_cols == (coo.cols // 2 + 1 + 3) // 4 * 4
        assert res.ms > 0
        got = res.d_output.cpu().numpy()[:, : coo.cols // 2 + 1]
        assert fp64.rel_l2(got, ref) < REL_L2_TOL
    with pytest.raises(RuntimeError):
        gb.sparse_fft_csc_bluestein_mixed_radix(coo, 0)


@pytest.mark.parametrize("policy", [gb.GBSP_LEN_3SMOOTH, gb.GBSP_LEN_7SMOOTH, gb.GBSP_LEN_POW2])
@pytest.mark.parametrize("shape", [(64, 64, 400), (101, 127, 900), (300, 257, 3000), (211, 1000, 4000)])
def test_against_reference_gpu_method_port(cuda, policy, shape):
    # the FP32 restatement of the reference's own method on the same input:
    # rel-L2 <= 1e-5 between the two FP32 forms
    from oracle import ref_port
    g = np.random.default_rng(shape[0] + shape[1])
    coo = synthetic.normalise(shape[0], shape[1], g.integers(0, shape[0], shape[2]),
                              g.integers(0, shape[1], shape[2]))
    got, _ = run_plan(coo, length_policy=policy)
    port = ref_port.reference_gpu_method(coo.rows, coo.cols, coo.row_idx, coo.col_idx, policy)
    assert fp64.rel_l2(got[:, : coo.cols // 2 + 1], port) <= REL_L2_TOL


def test_uniform_3001x2048_vs_reference_port(cuda):
    from oracle import ref_port
    coo = synthetic.config_matrix("uniform_3001x2048")
    got, _ = run_plan(coo, length_policy=gb.GBSP_LEN_3SMOOTH)
    port = ref_port.reference_gpu_method(coo.rows, coo.cols, coo.row_idx, coo.col_idx, 3)
    assert fp64.rel_l2(got[:, : coo.cols // 2 + 1], port) <= REL_L2_TOL


def test_cli_methods_with_host_reference(cuda, tmp_path):
    # the reference-compatible driver end to end: read .mtx, run both hot
    # methods, the graph replay and the power-of-two methods (direct and
    # streamed), check lines against the FP64 host spectrum
    import subprocess
    from cuspfft_gb300 import build
    coo = synthetic.uniform_matrix(97, 130, 900, seed=31)
    path = tmp_path / "m.mtx"
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern general\n")
        f.write(f"{coo.rows} {coo.cols} {coo.nnz}\n")
        for r, c in zip(coo.row_idx, coo.col_idx):
            f.write(f"{r + 1} {c + 1}\n")
    exe = build.build().parent / "cuspfft_gb300"
    res = subprocess.run([str(exe), str(path), "--sparse-only", "--cpu-reference", "--csc-mixed-radix",
                          "--csc-cufft-smooth", "--csc-mixed-radix-graph", "--csc-stockham-smem",
                          "--csc-stockham-cufft", "--csc-stockham-cufft-stream", "--csc-binary-lut",
                          "--csc-binary-stockham-smem", "--csc-tile", "16", "--repeat", "3"],
                         capture_output=True, text=True, timeout=300)
    assert res.returncode == 0, res.stderr
    checks = [ln for ln in res.stdout.splitlines() if ln.strip().startswith("check")]
    assert len(checks) == 8, res.stdout
    for ln in checks:
        max_rel = float(ln.split("max_rel")[1].split()[0])
        assert max_rel < 1e-4, ln
    assert "n=3" in res.stdout


@pytest.mark.parametrize("rows,cols,index_bytes", [(60001, 40, 0), (70001, 64, 0), (131071, 33, 4)])
def test_tall_matrices_two_level_table(cuda, rows, cols, index_bytes):
    # too many rows for a full or half twiddle table in shared memory: pass 1
    # reads W^p as hi[p / 256] * lo[p % 256]; above 65535 rows the phases use
    # 64-bit products
    g = np.random.default_rng(rows)
    n = 3 * rows
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, n), g.integers(0, cols, n))
    got, info = run_plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, index_bytes=index_bytes)
    assert info["row_table_mode"] == 2
    us = np.unique(np.r_[0:4, rows // 3, rows // 2 - 1:rows // 2 + 2, rows - 3:rows] % rows)
    check_against_oracle(coo, got, us=us)


def test_two_level_table_on_request(cuda):
    coo = synthetic.uniform_matrix(3001, 2048, 30730, seed=1)
    full, _ = run_plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, row_table_mode=1)
    two, info = run_plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, row_table_mode=3)
    assert info["row_table_mode"] == 2 and info["pass1_shape"] in (7, 8)
    assert fp64.rel_l2(two, full) < 1e-6
    check_against_oracle(coo, two)


@pytest.mark.parametrize("rows,cols", [(33, 120001), (5, 200003)])
def test_wide_matrices_many_channels(cuda, rows, cols):
    # the convolution needs more channels than a cluster holds (L = 240100 and
    # 401408, channels of at most ~28k points):
    # one CTA runs them in turn
    g = np.random.default_rng(cols)
    n = 4 * cols
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, n), g.integers(0, cols, n))
    got, info = run_plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH)
    assert info["channels"] > 8 and info["channel_mode"] == 2
    check_against_oracle(coo, got)
    with pytest.raises(gb.GbspError):
        gb.Plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, channel_mode=1)


# L = 82944 (3-smooth) and 81000 (7-smooth) run as three channels of 27648 and
# 27000 points; a 24000-point cap keeps the five-channel form covered
@pytest.mark.parametrize("policy,max_len,channels", [(gb.GBSP_LEN_3SMOOTH, 0, 3), (gb.GBSP_LEN_7SMOOTH, 0, 3),
                                                     (gb.GBSP_LEN_7SMOOTH, 24000, 5)])
def test_config_40421_uint32_indices(cuda, policy, max_len, channels):
    # the largest configuration: 40421^2 power-law adjacency, ~351k nnz,
    # 4-byte row indices (the reference's int32 pass 1,
    # src/sparse_fft_bluestein.cu:334-364), 6.5 GB output; the convolution
    # runs as K sequential channels in one CTA per row.  Rows are sampled on
    # the device; the pad columns of every row are checked there too.
    import torch
    coo = synthetic.config_matrix("uniform_powerlaw_40421")
    g = np.random.default_rng(40421)
    us = np.unique(np.concatenate([[0, 1, 2, coo.rows // 2, coo.rows // 2 + 1, coo.rows - 1],
                                   g.integers(0, coo.rows, 14)]))
    fc = coo.cols // 2 + 1
    with gb.Plan(coo, length_policy=policy, index_bytes=4, max_channel_len=max_len) as plan:
        info = plan.info
        assert info["index_bytes"] == 4
        assert info["channels"] == channels and info["channel_mode"] == 2
        out = plan.empty_output()
        out.fill_(complex(7.0, 7.0))
        plan.execute(out)
        torch.cuda.synchronize()
        assert plan.error_flags() == 0
        got = out[torch.as_tensor(us, device=out.device)].cpu().numpy()
        assert bool((out[:, fc:] == 0).all())
        del out
    ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx, us)
    err = fp64.rel_l2(got[:, :fc], ref)
    assert err <= REL_L2_TOL, f"rel-L2 {err:.3e}"


@pytest.mark.parametrize("name", ["uniform_3001x2048", "banded_powerlaw_8219"])
def test_exact_phase_mode(cuda, name):
    # exact_phases=1: every pass-1 twiddle is the FP64-built table entry at its
    # exact integer phase (u*r) mod rows; the default reads the table every
    # 4th row and steps the recurrence between.  Both within 1e-5 of FP64,
    # with and without Kahan compensation.
    coo = synthetic.config_matrix(name)
    us = None if coo.rows < 4000 else np.unique(np.r_[0, 1, 2, 3, 4, 5, 31, 32, 33, coo.rows // 2, coo.rows - 1])
    errs = {}
    for exact in (0, 1):
        for kahan in (0, -1):
            got, info = run_plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, exact_phases=exact,
                                 kahan_min_degree=kahan)
            assert info["exact_phases"] == exact
            errs[exact, kahan] = check_against_oracle(coo, got, us=us)
    print(name, {k: f"{v:.3e}" for k, v in errs.items()})


@pytest.mark.parametrize("rows,cols,index_bytes", [(24001, 40, 0), (70001, 64, 0)])
def test_exact_phase_mode_tall(cuda, rows, cols, index_bytes):
    # half table (24001 rows) and two-level table with 64-bit phases (70001)
    g = np.random.default_rng(rows + 1)
    n = 2 * rows
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, n), g.integers(0, cols, n))
    got, info = run_plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, exact_phases=1, index_bytes=index_bytes)
    us = np.unique(np.r_[0:5, rows // 2 - 1:rows // 2 + 2, rows - 3:rows] % rows)
    check_against_oracle(coo, got, us=us)


def test_exact_phase_mode_batch(cuda):
    import torch
    mats = [synthetic.uniform_matrix(r, c, n, seed=r) for r, c, n in [(501, 300, 4000), (1301, 977, 20000),
                                                                        (64, 2000, 900)]]
    with gb.Batch(mats, exact_phases=1) as batch:
        outs = batch.empty_outputs()
        batch.set_outputs(outs)
        batch.execute()
        torch.cuda.synchronize()
        assert batch.error_flags() == 0
        for coo, out in zip(mats, outs):
            check_against_oracle(coo, out.cpu().numpy())


@pytest.mark.parametrize("shape", [1, 2, 3, 4, 5, 6])
def test_every_pass1_shape(cuda, shape):
    # every pass-1 shape (rows per item, window width 16 / 32 / 64, full or
    # half table) gives the same spectrum within 1e-5 of FP64, including a
    # window with a heavy column split across tasks
    g = np.random.default_rng(shape)
    rows, cols = 2003, 1500
    r = np.concatenate([g.integers(0, rows, 30000), g.integers(0, rows, 1200)])
    c = np.concatenate([g.integers(0, cols, 30000), np.full(1200, 37)])
    coo = synthetic.normalise(rows, cols, r, c)
    got, info = run_plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, pass1_shape=shape)
    assert info["pass1_shape"] == shape
    check_against_oracle(coo, got)


@pytest.mark.parametrize("policy,cols", [(gb.GBSP_LEN_7SMOOTH, 2048), (gb.GBSP_LEN_7SMOOTH, 1029),
                                         (gb.GBSP_LEN_7SMOOTH, 375), (gb.GBSP_LEN_3SMOOTH, 243),
                                         (gb.GBSP_LEN_3SMOOTH, 1536), (gb.GBSP_LEN_POW2, 256),
                                         (gb.GBSP_LEN_7SMOOTH, 2), (gb.GBSP_LEN_7SMOOTH, 7),
                                         (gb.GBSP_LEN_7SMOOTH, 25000), (gb.GBSP_LEN_7SMOOTH, 25725),
                                         (gb.GBSP_LEN_3SMOOTH, 26244)])
def test_direct_row_fft(cuda, policy, cols):
    # cols already smooth for the policy: each row is one forward FFT of
    # length cols (fft_len = cols), the same DFT as the Bluestein convolution
    # that force_bluestein restores; odd lengths included (the row buffer is
    # padded to even for the bulk copy)
    g = np.random.default_rng(cols)
    rows = 301
    n = min(max(1, rows * cols // 20), 60000)
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, n), g.integers(0, cols, n))
    got, info = run_plan(coo, length_policy=policy)
    assert info["direct"] == 1 and info["fft_len"] == cols and info["channels"] == 1
    check_against_oracle(coo, got)
    blu, binfo = run_plan(coo, length_policy=policy, force_bluestein=1)
    assert binfo["direct"] == 0 and binfo["fft_len"] >= 2 * cols - 1
    check_against_oracle(coo, blu)
    assert fp64.rel_l2(got, blu) < 1e-5

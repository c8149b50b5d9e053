"""Parity with the reference's own GPU methods, run on the same GPU.

oracle/refgpu.py launches the reference's kernels (compiled for sm_103a from
its src/sparse_fft_bluestein.cu into oracle/_ref/ref_kernels.fatbin) in the
order its host code does for sparse_fft_csc_bluestein_mixed_radix
(src/sparse_fft_bluestein.cu:2256-2392) and
sparse_fft_csc_bluestein_cufft_smooth (:2557-2719).

Bars:
  * this library vs the reference's GPU output: rel-L2 <= 1e-5 (FP32 vs FP32)
  * each side vs the FP64 oracle: this library <= 1e-5; the reference's
    figure is stated (printed), and bounded loosely
  * the FP32 CPU restatement of the reference method (oracle/ref_gpu_port.c)
    vs the reference's GPU output: rel-L2 <= 1e-5
Skipped where the reference kernels were not built (no reference tree when
oracle/_ref was prepared).
"""
import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import synthetic
from oracle import fp64, refgpu

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not refgpu.available(), reason="reference kernels not built (oracle/_ref)")]

REL_L2_TOL = 1e-5
METHODS = {3: gb.GBSP_LEN_3SMOOTH, 7: gb.GBSP_LEN_7SMOOTH}


def ours(coo, policy):
    import torch
    with gb.Plan(coo, length_policy=policy) as plan:
        out = plan.empty_output()
        out.fill_(complex(7.0, 7.0))
        plan.execute(out)
        torch.cuda.synchronize()
        assert plan.error_flags() == 0
        return out.cpu().numpy()[:, : coo.cols // 2 + 1]


def sample_rows(rows, n=12, seed=0):
    g = np.random.default_rng(seed)
    return np.unique(np.concatenate([[0, 1, rows // 2, rows - 1], g.integers(0, rows, n)]))


@pytest.mark.parametrize("method", [3, 7])
def test_uniform_3001x2048_full_spectrum(cuda, method):
    coo = synthetic.config_matrix("uniform_3001x2048")
    ref, _ = refgpu.run(coo.rows, coo.cols, coo.row_idx, coo.col_idx, method, u_tile=128)
    got = ours(coo, METHODS[method])
    exact = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    e_pair, e_ours, e_ref = fp64.rel_l2(got, ref), fp64.rel_l2(got, exact), fp64.rel_l2(ref, exact)
    print(f"3001x2048 method {method}: ours vs reference GPU {e_pair:.3e}; vs FP64: ours {e_ours:.3e}, "
          f"reference {e_ref:.3e}")
    assert e_pair <= REL_L2_TOL
    assert e_ours <= REL_L2_TOL
    assert e_ref <= 1e-4


@pytest.mark.parametrize("method", [3, 7])
def test_banded_powerlaw_8219(cuda, method):
    coo = synthetic.config_matrix("banded_powerlaw_8219")
    ref, times = refgpu.run(coo.rows, coo.cols, coo.row_idx, coo.col_idx, method, u_tile=1024)
    got = ours(coo, METHODS[method])
    us = sample_rows(coo.rows)
    exact = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx, us)
    e_pair = fp64.rel_l2(got, ref)
    e_ours, e_ref = fp64.rel_l2(got[us], exact), fp64.rel_l2(ref[us], exact)
    print(f"8219^2 method {method}: ours vs reference GPU {e_pair:.3e} (whole spectrum); vs FP64 on "
          f"{us.size} rows: ours {e_ours:.3e}, reference {e_ref:.3e}; reference tile loop {times[0]:.2f} ms")
    assert e_pair <= REL_L2_TOL
    assert e_ours <= REL_L2_TOL
    assert e_ref <= 1e-4


@pytest.mark.parametrize("method", [3, 7])
@pytest.mark.parametrize("rows,cols,nnz", [(64, 64, 400), (101, 127, 900), (300, 257, 3000), (997, 13, 2000),
                                           (211, 1000, 4000)])
def test_random_shapes_and_port(cuda, method, rows, cols, nnz):
    from oracle import ref_port
    g = np.random.default_rng(rows * 7 + cols)
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, nnz), g.integers(0, cols, nnz))
    ref, _ = refgpu.run(coo.rows, coo.cols, coo.row_idx, coo.col_idx, method, u_tile=64)
    got = ours(coo, METHODS[method])
    port = ref_port.reference_gpu_method(coo.rows, coo.cols, coo.row_idx, coo.col_idx, method)
    assert fp64.rel_l2(got, ref) <= REL_L2_TOL
    # the CPU restatement of the reference method against its real GPU output
    assert fp64.rel_l2(port, ref) <= REL_L2_TOL


def test_wide_rows_int32_kernel(cuda):
    # cols > 65536: the reference uploads int32 indices and runs its unpacked
    # pass-1 kernel (src/sparse_fft_bluestein.cu:334-364); u*r < 2^32 here, so
    # its phases are exact and the two agree
    g = np.random.default_rng(70001)
    rows, cols, n = 33, 70001, 200_000
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, n), g.integers(0, cols, n))
    ref, _ = refgpu.run(coo.rows, coo.cols, coo.row_idx, coo.col_idx, 7, u_tile=33)
    got = ours(coo, gb.GBSP_LEN_7SMOOTH)
    assert fp64.rel_l2(got, ref) <= REL_L2_TOL


def test_tall_rows_reference_phase_overflow(cuda):
    # rows > 65536: the reference's phase_idx forms u*r in 32 bits
    # (include/sparse_fft_internal.cuh:51-53), which wraps once u*r >= 2^32,
    # so its spectrum leaves the definition; this library reduces the 64-bit
    # product and stays within 1e-5 of the FP64 oracle
    g = np.random.default_rng(3)
    rows, cols, n = 70001, 40, 30_000
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, n), g.integers(0, cols, n))
    ref, _ = refgpu.run(coo.rows, coo.cols, coo.row_idx, coo.col_idx, 7, u_tile=4096)
    got = ours(coo, gb.GBSP_LEN_7SMOOTH)
    us = np.array([0, 1, 2, 61357, 65535, 65537, 70000])
    exact = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx, us)
    assert fp64.rel_l2(got[us], exact) <= REL_L2_TOL
    assert fp64.rel_l2(ref[us], exact) > 1e-2

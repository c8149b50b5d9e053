"""The oracles themselves: the FP64 definition against independent
evaluations and known answers, and the FP32 restatement of the reference's
GPU methods against the FP64 definition."""
import numpy as np
import pytest

from cuspfft_gb300 import synthetic
from oracle import fp64, ref_port


def rand_coo(rows, cols, n, seed):
    g = np.random.default_rng(seed)
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, n), g.integers(0, cols, n))
    return coo.rows, coo.cols, coo.row_idx, coo.col_idx


@pytest.mark.parametrize("shape", [(1, 1, 1), (5, 8, 10), (13, 7, 30), (32, 30, 200), (64, 97, 600)])
def test_fp64_matches_direct_and_dense(shape):
    rows, cols, r, c = rand_coo(*shape, seed=sum(shape))
    F = fp64.spectrum_rows_fp64(rows, cols, r, c)
    assert np.max(np.abs(F - fp64.direct_dft_fp64(rows, cols, r, c))) < 1e-9
    assert np.max(np.abs(F - fp64.spectrum_dense_fp64(rows, cols, r, c))) < 1e-9


def test_known_answers():
    rows, cols, r, c = rand_coo(40, 50, 300, 1)
    F = fp64.spectrum_rows_fp64(rows, cols, r, c)
    assert abs(F[0, 0] - r.size) < 1e-9                     # F[0][0] = nnz
    full = np.fft.fft(np.conj(F[:, 1: (cols + 1) // 2]), axis=0)  # Hermitian rows
    Fneg = fp64.spectrum_rows_fp64(rows, cols, r, c, (-np.arange(rows)) % rows)
    assert np.allclose(Fneg[:, 0], np.conj(F[:, 0]))        # F[-u][0] = conj F[u][0]
    # Parseval over the full (two-sided) spectrum: sum |F|^2 = rows*cols*nnz
    a = np.zeros((rows, cols))
    a[r, c] = 1
    assert abs(np.sum(np.abs(np.fft.fft2(a)) ** 2) - rows * cols * r.size) < 1e-6 * rows * cols * r.size
    del full


def test_hermitian_pass1_symmetry():
    rows, cols, r, c = rand_coo(31, 20, 100, 2)
    S = fp64.column_sums_fp64(rows, cols, r, c, np.arange(rows))
    assert np.allclose(S[(rows - np.arange(rows)) % rows], np.conj(S))


@pytest.mark.parametrize("method", [3, 7])
@pytest.mark.parametrize("shape", [(7, 5, 12), (64, 64, 400), (101, 127, 900), (300, 257, 3000)])
def test_reference_gpu_port_accuracy(method, shape):
    rows, cols, r, c = rand_coo(*shape, seed=shape[0])
    got = ref_port.reference_gpu_method(rows, cols, r, c, method)
    ref = fp64.spectrum_rows_fp64(rows, cols, r, c)
    assert fp64.rel_l2(got, ref) < 1e-5


def test_cpu_path_restatement():
    rows, cols, r, c = rand_coo(33, 40, 200, 4)
    out, ms = ref_port.cpu_fft_r2c_2d(rows, cols, r, c)
    assert out.shape == (rows, cols // 2 + 1) and ms >= 0
    assert fp64.rel_l2(out, fp64.spectrum_rows_fp64(rows, cols, r, c)) < 1e-5

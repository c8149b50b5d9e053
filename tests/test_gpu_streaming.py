"""Streaming the spectrum to host memory (gbsp_execute_to_host; the
reference's sparse_fft_csc_stockham_streaming / _cufft_streaming).

Tiles whose starts are multiples of 256 Bluestein rows see the same pass-1
work items as the one-shot transform, so their output is bit-identical to
Plan.execute; other tile sizes must agree with the FP64 oracle within the
usual rel-L2 1e-5.  Even and odd row counts cover the self-mirrored middle
row and its absence."""
import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import synthetic
from oracle import fp64

pytestmark = pytest.mark.gpu


def device_result(coo, **kw):
    import torch
    with gb.Plan(coo, **kw) as p:
        out = p.empty_output()
        p.execute(out)
        torch.cuda.synchronize()
        return out.cpu().numpy()


def streamed(coo, tile, pinned=True, **kw):
    import torch
    with gb.Plan(coo, **kw) as p:
        host = torch.full((coo.rows, p.output_pitch), complex(5.0, 5.0), dtype=torch.complex64)
        if pinned:
            host = host.pin_memory()
        p.execute_to_host(host, tile_rows=tile)
        assert p.error_flags() == 0
        return host.numpy().copy()


@pytest.mark.parametrize("rows,cols", [(1, 9), (2, 2), (255, 300), (256, 301), (1025, 777), (2048, 1000)])
@pytest.mark.parametrize("tile", [1, 7, 100, 256, 1024])
def test_streaming_matches_oracle(cuda, rows, cols, tile):
    g = np.random.default_rng(rows * 7 + cols)
    coo = synthetic.normalise(rows, cols, g.integers(0, rows, max(1, rows * cols // 50)),
                              g.integers(0, cols, max(1, rows * cols // 50)))
    got = streamed(coo, tile, length_policy=gb.GBSP_LEN_7SMOOTH)
    fc = cols // 2 + 1
    ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    assert fp64.rel_l2(got[:, :fc], ref) <= 1e-5
    assert np.all(got[:, fc:] == 0)


@pytest.mark.parametrize("policy", [gb.GBSP_LEN_3SMOOTH, gb.GBSP_LEN_7SMOOTH])
def test_streaming_bit_identical_on_256_row_tiles(cuda, policy):
    coo = synthetic.uniform_matrix(3001, 2048, 30730, seed=1)
    want = device_result(coo, length_policy=policy)
    for tile in (256, 1024):
        assert np.array_equal(streamed(coo, tile, length_policy=policy), want)
    assert np.array_equal(streamed(coo, 512, pinned=False, length_policy=policy), want)


@pytest.mark.parametrize("channel_mode", [1, 2])
def test_streaming_cluster_plan(cuda, channel_mode):
    # convolution split over 3 channels (clusters, or sequential in one CTA)
    coo = synthetic.uniform_matrix(700, 333, 5000, seed=4)
    got = streamed(coo, 64, length_policy=gb.GBSP_LEN_7SMOOTH, max_channel_len=250, channel_mode=channel_mode)
    ref = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    assert fp64.rel_l2(got[:, :coo.cols // 2 + 1], ref) <= 1e-5


def test_streaming_rejects_bad_arguments(cuda):
    import torch
    coo = synthetic.uniform_matrix(64, 64, 200, seed=2)
    with gb.Plan(coo) as p:
        with pytest.raises(ValueError):
            p.execute_to_host(torch.zeros((64, p.output_pitch), dtype=torch.complex64, device="cuda"))
        with pytest.raises(gb.GbspError):
            p.execute_to_host(torch.zeros((64, 1), dtype=torch.complex64))


def test_cli_streaming_methods(cuda, tmp_path):
    import subprocess
    from cuspfft_gb300 import build
    coo = synthetic.uniform_matrix(301, 250, 2000, seed=33)
    path = tmp_path / "m.mtx"
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern general\n")
        f.write(f"{coo.rows} {coo.cols} {coo.nnz}\n")
        for r, c in zip(coo.row_idx, coo.col_idx):
            f.write(f"{r + 1} {c + 1}\n")
    exe = build.build().parent / "cuspfft_gb300"
    res = subprocess.run([str(exe), str(path), "--sparse-only", "--cpu-reference", "--csc-stockham-stream",
                          "--csc-stockham-cufft-stream", "--csc-tile", "40"], capture_output=True, text=True,
                         timeout=300)
    assert res.returncode == 0, res.stderr
    assert "Sparse CSC (cufft stream)" in res.stdout and "Sparse CSC (Stockham strm)" in res.stdout
    checks = [ln for ln in res.stdout.splitlines() if ln.strip().startswith("check")]
    assert len(checks) == 2, res.stdout
    for ln in checks:
        assert float(ln.split("max_rel")[1].split()[0]) < 1e-4, ln


def test_streaming_with_reserved_slabs(cuda):
    import torch
    coo = synthetic.uniform_matrix(1025, 777, 8000, seed=6)
    want = streamed(coo, 256, length_policy=gb.GBSP_LEN_7SMOOTH)
    with gb.Plan(coo, length_policy=gb.GBSP_LEN_7SMOOTH, stream_tile_rows=256) as p:
        host = torch.zeros((coo.rows, p.output_pitch), dtype=torch.complex64).pin_memory()
        for _ in range(2):  # the second call reuses the slabs and the copy stream
            host.fill_(complex(9.0, 9.0))
            p.execute_to_host(host, tile_rows=256)
            assert np.array_equal(host.numpy(), want)
        p.execute_to_host(host, tile_rows=1024)  # larger tiles than reserved: slabs reallocated
        assert fp64.rel_l2(host.numpy(), want) < 1e-6

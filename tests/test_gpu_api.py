"""The C++ drop-in API (include/sparse_fft.h) called directly from C++.

tests/cpp/api_dump.cpp links libgbspfft.so, runs one method on a Matrix
Market file several times in one process and dumps the last spectrum, which
is checked against the FP64 oracle (rel-L2 <= 1e-5).  Covers the CUDA-graph
entry point sparse_fft_csc_bluestein_mixed_radix_graph
(src/sparse_fft_bluestein.cu:2402-2549) with many captured tiles, and the
reference's memory metric, mem_bytes (src/sparse_fft_bluestein.cu:7-20), on
repeated calls.
"""
import re
import subprocess

import numpy as np
import pytest

import cuspfft_gb300 as gb
from cuspfft_gb300 import build, synthetic
from oracle import fp64

pytestmark = pytest.mark.gpu

REL_L2_TOL = 1e-5
ROOT = build.ROOT


@pytest.fixture(scope="module")
def api_dump(tmp_path_factory):
    lib = build.build()
    exe = tmp_path_factory.mktemp("api") / "api_dump"
    cmd = [build.nvcc(), "-std=c++17", "-O2", f"-I{ROOT / 'include'}", str(ROOT / "tests" / "cpp" / "api_dump.cpp"),
           "-o", str(exe), f"-L{lib.parent}", "-lgbspfft", f"-Xlinker=-rpath,{lib.parent}"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-3000:]
    return exe


def write_mtx(path, coo):
    with open(path, "w") as f:
        f.write("%%MatrixMarket matrix coordinate pattern general\n")
        f.write(f"{coo.rows} {coo.cols} {coo.nnz}\n")
        f.write("".join(f"{r + 1} {c + 1}\n" for r, c in zip(coo.row_idx, coo.col_idx)))


def run_dump(exe, tmp_path, coo, method, u_tile, repeat):
    mtx, out = tmp_path / "m.mtx", tmp_path / "out.bin"
    write_mtx(mtx, coo)
    r = subprocess.run([str(exe), method, str(mtx), str(u_tile), str(repeat), str(out)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    calls = [tuple(map(float, m)) for m in re.findall(r"ms (\S+) mem_bytes (\d+) output_cols (\d+)", r.stdout)]
    assert len(calls) == repeat
    raw = np.fromfile(out, dtype=np.int32, count=3)
    rows, cols, oc = map(int, raw)
    spec = np.fromfile(out, dtype=np.complex64, offset=12).reshape(rows, oc)
    return spec[:, : cols // 2 + 1], calls


@pytest.mark.parametrize("u_tile", [128, 1024])
def test_graph_entry_point(cuda, api_dump, tmp_path, u_tile):
    coo = synthetic.config_matrix("uniform_3001x2048")
    got, calls = run_dump(api_dump, tmp_path, coo, "mixed_radix_graph", u_tile, 2)
    exact = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    assert fp64.rel_l2(got, exact) <= REL_L2_TOL
    plain, _ = run_dump(api_dump, tmp_path, coo, "mixed_radix", u_tile, 1)
    assert np.array_equal(got, plain)  # the graph replays the same kernels
    assert all(c[0] > 0 for c in calls)


@pytest.mark.parametrize("method,policy", [("mixed_radix", gb.GBSP_LEN_3SMOOTH),
                                           ("cufft_smooth", gb.GBSP_LEN_7SMOOTH),
                                           ("mixed_radix_graph", gb.GBSP_LEN_3SMOOTH)])
def test_mem_bytes_on_repeated_calls(cuda, api_dump, tmp_path, method, policy):
    # every call reports the buffers it holds at its end -- the plan's device
    # memory and the output -- including calls whose plan memory the
    # library's pool hands out again
    coo = synthetic.uniform_matrix(1201, 900, 20000, seed=4)
    got, calls = run_dump(api_dump, tmp_path, coo, method, 64, 3)
    mems = [int(c[1]) for c in calls]
    with gb.Plan(coo, length_policy=policy, u_tile=64) as plan:
        expect = plan.device_bytes + coo.rows * plan.output_pitch * 8
    assert mems == [expect] * 3
    exact = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    assert fp64.rel_l2(got, exact) <= REL_L2_TOL


def test_streaming_entry_point(cuda, api_dump, tmp_path):
    coo = synthetic.uniform_matrix(777, 1500, 9000, seed=6)
    got, calls = run_dump(api_dump, tmp_path, coo, "stockham_streaming", 100, 2)
    exact = fp64.spectrum_rows_fp64(coo.rows, coo.cols, coo.row_idx, coo.col_idx)
    assert fp64.rel_l2(got, exact) <= REL_L2_TOL
    assert calls[0][1] == calls[1][1] > 0


def test_cli_repeat_reports_the_first_calls_memory(cuda, tmp_path):
    # the reference driver's --repeat N (1 warm-up + N timed calls) prints the
    # last call's mem_bytes; it must equal a single call's
    exe = build.build().parent / "cuspfft_gb300"
    coo = synthetic.uniform_matrix(501, 640, 6000, seed=8)
    path = tmp_path / "m.mtx"
    write_mtx(path, coo)
    mb = {}
    for rep in (1, 3):
        r = subprocess.run([str(exe), str(path), "--sparse-only", "--csc-mixed-radix", "--csc-cufft-smooth",
                            "--csc-tile", "64", "--repeat", str(rep)], capture_output=True, text=True, timeout=300)
        assert r.returncode == 0, r.stderr
        rows = re.findall(r"^Sparse CSC \((?:mixed-radix|cufft smooth)\)\s+\S+\s+(\S+)", r.stdout, re.M)
        assert len(rows) == 2, r.stdout
        mb[rep] = [float(x) for x in rows]
    assert mb[1] == mb[3] and all(v > 0 for v in mb[1])

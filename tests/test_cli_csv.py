"""The CLI's stdout parses into the reference's CSV rows (the formats its
scripts/parse_log.awk reads).  Runs on a log the CLI wrote on a GB300
(tests/golden/cli_run.log, regenerated by tests/golden/make_cli_log.sh) and on
a live run here without a GPU, where every method reports a failure row."""
import subprocess
from pathlib import Path

import pytest

from cli_log import parse_log

GOLDEN = Path(__file__).resolve().parent / "golden" / "cli_run.log"


def test_golden_log_parses():
    rows = parse_log(GOLDEN.read_text())
    by = {r["method"]: r for r in rows}
    for label in ("Sparse CSC (mixed-radix)", "Sparse CSC (cufft smooth)", "Sparse CSC (mr-graph)",
                  "Sparse CSC (cufft stream)", "Sparse CSC (Stockham strm)", "Sparse CSC (binary LUT)"):
        r = by[label]
        assert float(r["median_ms"]) > 0 and r["n_iters"] == "3"
        assert float(r["min_ms"]) <= float(r["median_ms"]) <= float(r["max_ms"])
        assert float(r["max_rel"]) < 1e-4, r
    assert by["CPU reference (FP64)"]["n_iters"] == "1"
    assert by["Dense cuFFT (baseline)"]["error"] == "not in this library"
    assert rows[0]["rows"] == "301" and rows[0]["cols"] == "250"


def test_failure_rows_without_gpu(tmp_path):
    from cuspfft_gb300 import build
    exe = build.build().parent / "cuspfft_gb300"
    mtx = Path(__file__).resolve().parent / "golden" / "mtx" / "pattern.mtx"
    res = subprocess.run([str(exe), str(mtx), "--csc-mixed-radix", "--csc-stockham-cufft-stream", "--spfft"],
                         capture_output=True, text=True, timeout=120)
    if res.returncode != 0:
        pytest.skip("CLI needs a CUDA runtime to start: " + res.stderr.strip()[:80])
    rows = parse_log(res.stdout)
    labels = [r["method"] for r in rows]
    assert "Dense cuFFT (baseline)" in labels and "--spfft" in labels
    assert all(r["median_ms"] != "" or r["error"] for r in rows)

"""Drop-in proof: the reference's own driver (src/main.cu) and dense baseline
compile against the reference's headers and link against libgbspfft.so in
place of its sparse_fft_bluestein.cu / mtx_reader.cu, then run its --help.
Needs the reference tree (present where the fixtures are generated); the
binary is built in a temporary directory, never in the repository."""
import os
import shutil
import subprocess
from pathlib import Path

import pytest

from cuspfft_gb300 import build


def reference_dir() -> Path:
    """GBSP_REFERENCE_DIR, else the tree oracle/build_ref.sh compiled from
    (recorded in oracle/_ref/REFERENCE_DIR); an empty path when neither is set."""
    env = os.environ.get("GBSP_REFERENCE_DIR")
    if env:
        return Path(env)
    rec = Path(__file__).resolve().parent.parent / "oracle" / "_ref" / "REFERENCE_DIR"
    return Path(rec.read_text().strip()) if rec.exists() else Path("/nonexistent")


REF = reference_dir()


@pytest.mark.skipif(not (REF / "src" / "main.cu").exists(), reason="reference sources not present")
@pytest.mark.skipif(shutil.which("nvcc") is None and not Path("/usr/local/cuda/bin/nvcc").exists(),
                    reason="nvcc not available")
def test_reference_driver_links_against_library(tmp_path):
    lib = build.build()
    nvcc = build.nvcc()
    exe = tmp_path / "cuSpFFT_on_gbsp"
    cmd = [nvcc, "-std=c++17", "-O1", "-w", "--expt-relaxed-constexpr", "-gencode",
           "arch=compute_103a,code=sm_103a", f"-I{REF / 'include'}", str(REF / "src" / "main.cu"),
           str(REF / "src" / "dense_baseline.cu"), "-o", str(exe), f"-L{lib.parent}", "-lgbspfft",
           f"-Xlinker=-rpath,{lib.parent}", "-lcufft"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    h = subprocess.run([str(exe), "--help"], capture_output=True, text=True, timeout=60)
    assert h.returncode == 0 and "--csc-mixed-radix" in h.stderr

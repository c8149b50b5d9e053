"""Builds the oracle's native helpers -- TEST INFRASTRUCTURE ONLY.

  oracle/_build/libref_port.so   gcc build of ref_gpu_port.c (the FP32 CPU
                                 restatement of the reference's GPU methods)
  oracle/_ref/libref_host.so     the reference's own host code compiled from
                                 its sources by build_ref.sh, only where the
                                 reference tree is present
"""
from __future__ import annotations

import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent


def build() -> None:
    out = HERE / "_build"
    out.mkdir(exist_ok=True)
    lib = out / "libref_port.so"
    src = HERE / "ref_gpu_port.c"
    if not lib.exists() or lib.stat().st_mtime < src.stat().st_mtime:
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", str(src), "-o", str(lib), "-lm"],
                       check=True)
    ref_dir = Path(os.environ.get("GBSP_REFERENCE_DIR", "/root/reference"))
    ref_lib = HERE / "_ref" / "libref_host.so"
    if (ref_dir / "src").exists() and (not ref_lib.exists() or
                                        ref_lib.stat().st_mtime < (HERE / "ref_shim.cu").stat().st_mtime):
        subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True)


if __name__ == "__main__":
    build()

"""Builds the oracle's native helpers -- TEST INFRASTRUCTURE ONLY.

  oracle/_build/libref_port.so        gcc build of ref_gpu_port.c (the FP32 CPU
                                      restatement of the reference's GPU methods)
  oracle/_build/libref_gpu_driver.so  g++ build of ref_gpu_driver.cpp, the host
                                      side that launches the reference's own
                                      kernels (CUDA runtime, driver API, cuFFT)
  oracle/_ref/libref_host.so,         the reference's own host code and GPU
  oracle/_ref/ref_kernels.fatbin      kernels compiled from its sources by
                                      build_ref.sh, only where the reference
                                      tree is present (GBSP_REFERENCE_DIR, else
                                      the path build_ref.sh names); on a machine
                                      without it the prebuilt files are used
"""
from __future__ import annotations

import os
import shutil
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent


def _cuda_home() -> Path:
    nv = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return Path(nv).resolve().parent.parent


def _stale(target: Path, deps: list[Path]) -> bool:
    return not target.exists() or any(d.stat().st_mtime > target.stat().st_mtime for d in deps)


def build() -> None:
    out = HERE / "_build"
    out.mkdir(exist_ok=True)
    lib = out / "libref_port.so"
    src = HERE / "ref_gpu_port.c"
    if _stale(lib, [src]):
        subprocess.run(["gcc", "-O2", "-fPIC", "-shared", "-std=c11", str(src), "-o", str(lib), "-lm"],
                       check=True)
    drv = out / "libref_gpu_driver.so"
    drv_src = HERE / "ref_gpu_driver.cpp"
    if _stale(drv, [drv_src]):
        cuda = _cuda_home()
        libdirs = [p for p in (cuda / "lib64", cuda / "lib64" / "stubs", cuda / "lib", cuda / "lib" / "stubs")
                   if p.exists()]
        cmd = ["g++", "-O2", "-fPIC", "-shared", "-std=c++17", f"-I{cuda / 'include'}", str(drv_src),
               "-o", str(drv)] + [f"-L{p}" for p in libdirs] + ["-lcufft", "-lcudart", "-lcuda",
                                                                  f"-Wl,-rpath,{cuda / 'lib64'}"]
        subprocess.run(cmd, check=True)
    ref_dir = Path(os.environ.get("GBSP_REFERENCE_DIR", "/root/reference"))
    ref_out = [HERE / "_ref" / "libref_host.so", HERE / "_ref" / "ref_kernels.fatbin"]
    if (ref_dir / "src").exists() and any(_stale(t, [HERE / "ref_shim.cu", HERE / "build_ref.sh"])
                                          for t in ref_out):
        env = dict(os.environ, GBSP_REFERENCE_DIR=str(ref_dir))
        subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True, env=env)


if __name__ == "__main__":
    build()

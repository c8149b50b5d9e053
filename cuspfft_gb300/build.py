"""Builds the native parts of cuspfft_gb300 in-tree with nvcc / g++.

Outputs (all under cuspfft_gb300/_build/, git-ignored):
  libgbspfft.so     the C ABI (include/gbspfft.h) and the C++ drop-in API
                    (include/sparse_fft.h, include/mtx_reader.h)
  cuspfft_gb300     the command-line driver with the reference's flags

Only sm_103a code is generated.  Translation units compile in parallel so a
fresh build takes well under a minute.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              f"-I{INCLUDE}", f"-I{CSRC}"]

LIB_SOURCES = ["gbsp_rows_multi.cu", "gbsp_rows_seq.cu", "gbsp_rows.cu", "gbsp_pass1.cu", "gbsp_pass1_exact.cu",
               "gbsp_plan.cu", "gbsp_planner.cu", "gbsp_mlp.cu", "gbsp_host.cpp", "sparse_fft_api.cu"]
CLI_SOURCES = ["cli_main.cpp"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found")


def _run(cmd: list[str]) -> None:
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")


def _stale(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _deps() -> list[Path]:
    return sorted(CSRC.glob("*")) + sorted(INCLUDE.glob("*.h")) + [Path(__file__)]


def build(verbose: bool = False, force: bool = False) -> Path:
    """Compiles libgbspfft.so and the CLI; returns the library path."""
    BUILD.mkdir(parents=True, exist_ok=True)
    lib = BUILD / "libgbspfft.so"
    cli = BUILD / "cuspfft_gb300"
    deps = _deps()
    if not force and not _stale(lib, deps) and not _stale(cli, deps):
        return lib
    nv = nvcc()
    objs = []
    jobs = []
    for src in LIB_SOURCES:
        obj = BUILD / (Path(src).stem + ".o")
        objs.append(obj)
        lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
        jobs.append([nv, *NVCC_FLAGS, *ARCH, *lang, "-c", str(CSRC / src), "-o", str(obj)])
    cli_obj = BUILD / "cli_main.o"
    jobs.append([nv, *NVCC_FLAGS, "-x", "c++", "-c", str(CSRC / CLI_SOURCES[0]), "-o", str(cli_obj)])
    with cf.ThreadPoolExecutor(max_workers=min(len(jobs), os.cpu_count() or 4)) as ex:
        for fut in [ex.submit(_run, j) for j in jobs]:
            fut.result()
    tmp_lib = BUILD / "libgbspfft.so.tmp"
    _run([nv, *ARCH, "-shared", "-o", str(tmp_lib), *map(str, objs), "-lcudart_static", "-lrt", "-ldl",
          "-lpthread"])
    os.replace(tmp_lib, lib)
    _run([nv, *ARCH, "-o", str(cli), str(cli_obj), f"-L{BUILD}", "-lgbspfft",
          f"-Xlinker=-rpath,{BUILD}", "-Xlinker=-rpath,$ORIGIN"])
    if verbose:
        print(f"built {lib} and {cli}", file=sys.stderr)
    return lib


if __name__ == "__main__":
    build(verbose=True, force="--force" in sys.argv)

"""The command-line driver: flags and messages of the reference CLI
(src/main.cu:217-311).  Nothing here needs a GPU."""
import subprocess
from pathlib import Path

import pytest

from cuspfft_gb300 import build

CLI = build.BUILD / "cuspfft_gb300"
G = Path(__file__).resolve().parent / "golden" / "mtx"


@pytest.fixture(scope="module", autouse=True)
def built():
    build.build()


def run(*args):
    return subprocess.run([str(CLI), *map(str, args)], capture_output=True, text=True, timeout=120)


def test_help():
    r = run("--help")
    assert r.returncode == 0 and "--csc-mixed-radix" in r.stderr and "--csc-cufft-smooth" in r.stderr
    assert run().returncode == 1


def test_flag_errors():
    m = G / "pattern.mtx"
    assert "Unknown option: --bogus" in run(m, "--bogus").stderr
    assert "--csc-tile must be positive" in run(m, "--csc-tile", "0").stderr
    assert "--repeat requires an integer value" in run(m, "--repeat").stderr


def test_bad_file():
    r = run(G / "bad_header.mtx", "--sparse-only")
    assert r.returncode == 1 and "Not a Matrix Market file" in r.stderr

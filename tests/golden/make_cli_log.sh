#!/bin/sh
# Regenerates tests/golden/cli_run.log: the CLI on a seeded 301 x 250 matrix
# with every method it runs, 3 timed repeats and the FP64 host check.
# Needs a GPU; run from the repository root after the library is built.
set -e
python - <<'PY'
import sys
sys.path.insert(0, ".")
from cuspfft_gb300 import synthetic
coo = synthetic.uniform_matrix(301, 250, 2000, seed=33)
with open("/tmp/cli_run.mtx", "w") as f:
    f.write("%%MatrixMarket matrix coordinate pattern general\n")
    f.write(f"{coo.rows} {coo.cols} {coo.nnz}\n")
    for r, c in zip(coo.row_idx, coo.col_idx):
        f.write(f"{r + 1} {c + 1}\n")
PY
cuspfft_gb300/_build/cuspfft_gb300 /tmp/cli_run.mtx --cpu-reference --csc-mixed-radix --csc-cufft-smooth \
    --csc-mixed-radix-graph --csc-stockham-stream --csc-stockham-cufft-stream --csc-binary-lut \
    --csc-tile 64 --repeat 3 | sed 's|^Matrix: .*|Matrix: cli_run.mtx|' > "${1:-tests/golden/cli_run.log}"

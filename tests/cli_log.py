"""Parser of the CLI's stdout into the reference's CSV rows (test helper).

Restates scripts/parse_log.awk of the reference (:1-18 schema, four line
formats): repeat-mode and single-run timing rows, correctness-check rows
and failure rows, keyed by the same label canonicalisation (canon(): drop
" (baseline)" and parentheses, squeeze blanks).  The reference's sweep and
plot tooling reads exactly these rows, so a log that parses here parses
there."""
from __future__ import annotations

import re

FAIL = re.compile(r"^(.{26})  +OOM +OOM +\[(.*)\]$")
REPEAT = re.compile(r"^(.{26})  +([0-9.]+) +([0-9.]+) +\[min ([0-9.]+), max ([0-9.]+)\] +n=([0-9]+)")
SINGLE = re.compile(r"^(.{26})  +([0-9.]+) +([0-9.]+)(\s.*)?$")
CHECK = re.compile(r"^  check (.+)  +max_abs +([0-9.eE+-]+) +max_rel +([0-9.eE+-]+) +rms_abs +([0-9.eE+-]+)")


def canon(s: str) -> str:
    s = s.replace(" (baseline)", "")
    s = re.sub(r"[()]", "", s)
    s = re.sub(r"[ \t]+", " ", s)
    return s.strip()


def parse_log(text: str) -> list[dict]:
    meta = {"rows": "", "cols": "", "nnz": ""}
    order, timing, correct, errors = [], {}, {}, {}

    def record(method):
        if canon(method) not in [canon(m) for m in order]:
            order.append(method)

    for line in text.splitlines():
        if line.startswith("Size:"):
            f = line.split()
            meta["rows"], meta["cols"] = f[1], f[3]
            continue
        if line.startswith("nnz:"):
            meta["nnz"] = line.split()[1]
            continue
        m = FAIL.match(line)
        if m:
            method = m.group(1).rstrip()
            timing[canon(method)] = {"median_ms": "", "min_ms": "", "max_ms": "", "n_iters": "", "mem_mb": ""}
            errors[canon(method)] = m.group(2)
            record(method)
            continue
        m = REPEAT.match(line)
        if m:
            method = m.group(1).rstrip()
            timing[canon(method)] = {"median_ms": m.group(2), "min_ms": m.group(4), "max_ms": m.group(5),
                                     "n_iters": m.group(6), "mem_mb": m.group(3)}
            record(method)
            continue
        m = SINGLE.match(line)
        if m:
            method = m.group(1).rstrip()
            if canon(method) not in timing:
                timing[canon(method)] = {"median_ms": m.group(2), "min_ms": "", "max_ms": "", "n_iters": "1",
                                         "mem_mb": m.group(3)}
                record(method)
            continue
        m = CHECK.match(line)
        if m:
            correct[canon(m.group(1).rstrip())] = {"max_abs": m.group(2), "max_rel": m.group(3),
                                                    "rms_abs": m.group(4)}
    rows = []
    for method in order:
        k = canon(method)
        row = {"method": method, **meta, **timing[k]}
        row.update(correct.get(k, {"max_abs": "", "max_rel": "", "rms_abs": ""}))
        row["error"] = errors.get(k, "")
        rows.append(row)
    return rows

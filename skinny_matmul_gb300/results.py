"""Persistent results store: one JSON object per line (JSONL), replacing the reference's sqlite
bench database (benchdb.hpp) with the same key set (perf.cu:286-307: multype, device, types, M,
N, name, inplace, zerobeta, blockCount, K, time, flops, bw, ...), plus the (M, N) grids and the
roofline-utilisation map of benchmark_analyzer.py:84-139 as text (no plotting dependency).

    python -m skinny_matmul_gb300.results results.jsonl --multype TSMM --types f64 --value bw
    python -m skinny_matmul_gb300.results results.jsonl --roofline 6707.2 1190 --types f64
"""
from __future__ import annotations

import argparse
import json
import os
import time
from typing import Iterable

KEYS = ("multype", "device", "types", "M", "N", "name", "inplace", "zerobeta", "K", "time", "flops", "bw")


def record(path: str, row: dict) -> dict:
    """Append one result (missing keys of KEYS raise); returns the stored object."""
    missing = [k for k in KEYS if k not in row]
    if missing:
        raise ValueError(f"result without {missing}")
    obj = dict(row)
    obj.setdefault("stamp", time.strftime("%Y-%m-%dT%H:%M:%S"))
    with open(path, "a") as f:
        f.write(json.dumps(obj, sort_keys=True) + "\n")
    return obj


def load(path: str, **where) -> list[dict]:
    """All results matching every key=value of `where` (later lines last)."""
    if not os.path.exists(path):
        return []
    out = []
    with open(path) as f:
        for ln in f:
            ln = ln.strip()
            if not ln:
                continue
            obj = json.loads(ln)
            if all(obj.get(k) == v for k, v in where.items()):
                out.append(obj)
    return out


def grid(rows: Iterable[dict], value: str, m_max: int = 64, n_max: int = 64) -> list[list[float | None]]:
    """g[n-1][m-1] = value of the latest result at (M, N) (None where there is none)."""
    g: list[list[float | None]] = [[None] * m_max for _ in range(n_max)]
    for r in rows:
        m, n = int(r["M"]), int(r["N"])
        if 1 <= m <= m_max and 1 <= n <= n_max:
            g[n - 1][m - 1] = float(r[value])
    return g


def roofline_grid(rows: Iterable[dict], stream_bw: float, peak_flops: float, m_max: int = 64,
                  n_max: int = 64) -> list[list[float | None]]:
    """max(bw / stream_bw, flops / peak) per (M, N), as benchmark_analyzer.py's roofline map
    (bw in GB/s, flops in GFLOP/s, the peaks in the same units)."""
    rows = list(rows)
    bw = grid(rows, "bw", m_max, n_max)
    fl = grid(rows, "flops", m_max, n_max)
    return [[None if b is None else max(b / stream_bw, (f or 0.0) / peak_flops) for b, f in zip(rb, rf)]
            for rb, rf in zip(bw, fl)]


_SHADES = " .:-=+*#%@"


def render(g: list[list[float | None]], lo: float | None = None, hi: float | None = None) -> str:
    """Text heat map, N upwards and M to the right; empty cells blank, ten shades from lo to hi."""
    vals = [v for row in g for v in row if v is not None]
    if not vals:
        return "(no results)"
    lo = min(vals) if lo is None else lo
    hi = max(vals) if hi is None else hi
    span = (hi - lo) or 1.0
    lines = []
    for n in range(len(g), 0, -1):
        row = g[n - 1]
        if all(v is None for v in row):
            continue
        cells = "".join(" " if v is None else _SHADES[min(9, max(0, int((v - lo) / span * 9.999)))] for v in row)
        lines.append(f"N={n:3d} |{cells}|")
    lines.append(f"      M=1..{len(g[0])}   shades ' '..'@' = {lo:.4g}..{hi:.4g}")
    return "\n".join(lines)


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("path")
    ap.add_argument("--multype")
    ap.add_argument("--types")
    ap.add_argument("--name")
    ap.add_argument("--value", default="bw")
    ap.add_argument("--roofline", nargs=2, type=float, metavar=("STREAM_GBS", "PEAK_GFLOPS"))
    a = ap.parse_args(argv)
    where = {k: v for k, v in (("multype", a.multype), ("types", a.types), ("name", a.name)) if v is not None}
    rows = load(a.path, **where)
    g = roofline_grid(rows, *a.roofline) if a.roofline else grid(rows, a.value)
    print(render(g, 0.0 if a.roofline else None, 1.0 if a.roofline else None))
    return 0


if __name__ == "__main__":
    raise SystemExit(main())

"""CPU tests of the JSONL results store (the replacement of the reference's sqlite bench DB)."""
import json

import pytest

from skinny_matmul_gb300 import results


def row(m, n, bw, flops=0.0, types="f64", multype="TSMM"):
    return {"multype": multype, "device": "GB300", "types": types, "M": m, "N": n, "name": "gb300-auto",
            "inplace": 0, "zerobeta": 0, "K": 1 << 20, "time": 1e-3, "flops": flops, "bw": bw}


def test_record_load_filter_and_grid(tmp_path):
    p = str(tmp_path / "r.jsonl")
    results.record(p, row(1, 1, 5000.0))
    results.record(p, row(2, 2, 4000.0))
    results.record(p, row(2, 2, 4200.0))  # later result wins in the grid
    results.record(p, row(4, 4, 100.0, types="c64"))
    rows = results.load(p, types="f64")
    assert len(rows) == 3 and all(json.loads(json.dumps(r)) == r for r in rows)
    g = results.grid(rows, "bw", 4, 4)
    assert g[0][0] == 5000.0 and g[1][1] == 4200.0 and g[3][3] is None
    text = results.render(g)
    assert "N=  2" in text and "N=  3" not in text


def test_roofline_grid_takes_the_larger_fraction(tmp_path):
    p = str(tmp_path / "r.jsonl")
    results.record(p, row(8, 8, 1400.0, flops=1050.0))
    g = results.roofline_grid(results.load(p), 6707.2, 1190.0, 8, 8)
    assert g[7][7] == pytest.approx(1050.0 / 1190.0)
    assert "@" in results.render(g, 0.0, 1.0) or "%" in results.render(g, 0.0, 1.0)


def test_missing_keys_rejected(tmp_path):
    with pytest.raises(ValueError):
        results.record(str(tmp_path / "r.jsonl"), {"M": 1})

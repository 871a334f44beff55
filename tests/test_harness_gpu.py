"""The sweep harness (the counterpart of the reference's script/ pipeline)
writes one CSV row per (engine, stencil, precision, mesh size)."""
import csv

import pytest

from tcstencil_gb300 import harness

pytestmark = pytest.mark.gpu


def test_harness_writes_rows(tcs, torch_cuda, tmp_path):
    out = tmp_path / "sweep.csv"
    assert harness.main(["--engines", "tensor,cudacore", "--stencils", "star2d1r,box2d2r",
                         "--precisions", "f16,split", "--sizes", "160,480", "--launches", "3",
                         "--csv", str(out)]) == 0
    rows = list(csv.DictReader(open(out)))
    # tensor: 2 precisions; cudacore: f16 only (no split) -> 3 x 2 stencils x 2 sizes
    assert len(rows) == 12
    for r in rows:
        assert float(r["gpts"]) > 0 and float(r["time_ms"]) > 0
        assert r["tile"] == "128x128" and int(r["steps"]) == 3
        assert int(r["kernel_launches"]) in (1, 3)
    assert {r["variant"] for r in rows} == {"tensor", "cudacore"}


def test_harness_tile_axis_marks_the_best_tile(tcs, torch_cuda, tmp_path):
    """--tiles sweeps the tile width of plain FP16 tensor sweeps, as the
    reference sweeps TILE_SIZE (script/param.py:5); one row per width, and
    exactly one best-tile row per configuration (script/process_data.py:29-43)."""
    out = tmp_path / "tiles.csv"
    assert harness.main(["--engines", "tensor,cudacore", "--stencils", "box2d1r",
                         "--precisions", "f16", "--sizes", "1024", "--launches", "3",
                         "--tiles", "128,96,64", "--csv", str(out)]) == 0
    rows = list(csv.DictReader(open(out)))
    tensor = [r for r in rows if r["variant"] == "tensor"]
    assert sorted(r["tile"] for r in tensor) == ["128x128", "128x64", "128x96"]
    assert sum(int(r["best_tile"]) for r in tensor) == 1
    cc = [r for r in rows if r["variant"] == "cudacore"]
    assert len(cc) == 1 and cc[0]["tile"] == "128x128" and cc[0]["best_tile"] == "1"

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

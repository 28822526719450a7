"""GPU test of the command line (the reference program's main(), main.cpp:275-284):
scene XML in, output.txt in the reference's format and a JSON run record out."""
import json
from pathlib import Path

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SCENES = Path(__file__).resolve().parent / "golden" / "scenes"


@pytest.mark.parametrize("precision", ["exact", "mixed"])
def test_cli_writes_output_and_record(built_lib, tmp_path, precision):
    from rayfactorcl_gb300.__main__ import main
    out, rec = tmp_path / "output.txt", tmp_path / "run.json"
    assert main([str(SCENES / "gen_enclosure3.xml"), "-o", str(out), "--record", str(rec),
                 "--precision", precision]) == 0
    rows = [r for r in out.read_text().splitlines() if r.strip()]
    assert len(rows) == 3 and all(r.endswith(",") for r in rows)
    F = np.array([[float(v) for v in r.rstrip(",").split(",")] for r in rows])
    r = json.loads(rec.read_text())
    assert r["surfaces"] == 3 and r["rays"] > 0 and r["kernel_ms"] > 0
    assert r["precision"] == precision
    # a closed enclosure: every ray of a row that was shot hits a surface, except the
    # few that meet a surface nearer than the reference's EPS = 1e-3 at the rims
    # (RayFactorGPU.cl:7) and leave through the crack
    shot = np.isfinite(F).all(axis=1) & (np.nan_to_num(F).sum(axis=1) > 0)
    err = float(np.abs(F[shot].sum(axis=1) - 1.0).max())
    assert err < 2e-3
    assert abs(r["max_row_sum_error"] - err) < 1e-6

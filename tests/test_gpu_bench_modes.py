"""bench.py's sweep modes on a small workload (16 disk charts): one JSON line per setting, and
the UVs of every setting equal to the first one's, bit for bit -- the settings swept here are
bit-identical by construction: upload parts and copy grids move the same bytes; the V(1,1)
cycle's rows are computed row by row whatever the tile rows; one lane sums its row in entry
order whatever its rows in flight."""
import json
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _run(args):
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--workload", "disks16", "--steps", "2",
                          "--warmup", "1", *args], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    return [json.loads(l) for l in out.stdout.splitlines() if l.startswith("{")]


def test_e2e_sweep_lines_and_bitwise_uvs():
    lines = _run(["--e2e-sweep", "RUV_UPLOAD_PARTS=8,RUV_H2D_GRID=38;RUV_UPLOAD_PARTS=3,RUV_H2D_GRID=152;"
                                 "RUV_H2D_KERNEL=0"])
    sweep = [l for l in lines if "setting" in l]
    assert [l["setting"] for l in sweep] == [{"RUV_UPLOAD_PARTS": "8", "RUV_H2D_GRID": "38"},
                                             {"RUV_UPLOAD_PARTS": "3", "RUV_H2D_GRID": "152"},
                                             {"RUV_H2D_KERNEL": "0"}]
    for l in sweep:
        assert l["uv_equal_to_first"] is True
        assert l["wall_ms_median"] > 0 and l["device_ms_median"] > 0
    assert lines[-1]["resident_device_ms_median"] > 0


def test_step_sweep_lines():
    lines = _run(["--step-sweep", "RUV_AMG_TILE=0;RUV_AMG_TILE=1024/256;RUV_AMG_L1SHAPE=0"])
    assert "spmv_shape_autotuned" in lines[0]
    sweep = [l for l in lines if "setting" in l]
    assert len(sweep) == 3
    for l in sweep:
        assert l["step_ms_median"] > 0
        assert l["cg_iters_max"] == sweep[0]["cg_iters_max"] > 0
        assert l["uv_max_abs_diff_to_first"] == 0.0

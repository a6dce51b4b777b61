"""bench.py's host-side pieces on the CPU: the settings of its sweep modes and its options."""
import os
import subprocess
import sys

import pytest

import bench

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_sweep_settings_parse():
    got = bench.sweep_settings("RUV_UPLOAD_PARTS=8,RUV_H2D_GRID=38;RUV_AMG_LANES=1/2/2/1; ;RUV_H2D_KERNEL=0")
    assert got == [{"RUV_UPLOAD_PARTS": "8", "RUV_H2D_GRID": "38"}, {"RUV_AMG_LANES": "1/2/2/1"},
                   {"RUV_H2D_KERNEL": "0"}]
    assert bench.sweep_settings("") == []
    assert bench.sweep_settings("A=x=y") == [{"A": "x=y"}]  # the value keeps every later '='
    with pytest.raises(ValueError):
        bench.sweep_settings("RUV_AMG_TILE")


def test_bench_lists_its_modes():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0, out.stderr
    for opt in ("--gpus", "--steps", "--warmup", "--impl", "--workload", "--e2e-sweep", "--step-sweep",
                "--no-autotune", "--ncu-step"):
        assert opt in out.stdout, opt

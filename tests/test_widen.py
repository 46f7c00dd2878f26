"""Integer widening of double-float values to FP64 (the FP32 thermalization's store):
the device code's host twin, compiled with the system C++ compiler and checked against
FP64 on a few million pairs."""
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parent.parent


def test_widen_df_within_one_ulp_and_float_is_its_rounding(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "widen_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "cudagfx_gb300" / "csrc"),
                    str(ROOT / "tests" / "widen_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "600000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "beyond one ulp 0" in r.stdout

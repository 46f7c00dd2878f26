"""FP64 <-> double-float conversions on the integer units: the widening of the FP32
thermalization's links to FP64 (gfx_widen.h) and the narrowing of FP64 fields into
float pairs for the rebased polish's base (gfx_narrow.h).  The device code's host twins,
compiled with the system C++ compiler and checked against FP64 on millions of values."""
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


def test_narrow_df_is_the_fp64_conversions_bit_for_bit(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "narrow_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "cudagfx_gb300" / "csrc"),
                    str(ROOT / "tests" / "narrow_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe), "300000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout

"""The float-float sine/cosine the float64 measurements use (ffmath.h) stays
within 8e-15 of the C library's float64 sin and cos on the host, over float
angles, exact differences of two angles, wide ranges and the floats nearest
multiples of pi/2."""

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_float_float_sincos_matches_float64(tmp_path):
    exe = tmp_path / "ffmath_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "gpu-monte-carlo_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "ffmath_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("OK")

"""The integer-only float32 uniform conversion equals the float64 route bit for bit."""

import subprocess
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]


def test_unit_f32_integer_rounding_matches_float64_route(tmp_path):
    exe = tmp_path / "unit_f32_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "gpu-monte-carlo_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "unit_f32_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("OK")


def test_integer_acceptance_threshold_equals_float_comparison(tmp_path):
    exe = tmp_path / "threshold_check"
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I", str(ROOT / "gpu-monte-carlo_gb300" / "csrc"),
                    str(ROOT / "tests" / "native" / "threshold_check.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip().endswith("OK")

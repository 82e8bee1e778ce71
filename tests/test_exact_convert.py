"""The exact float/int64/double conversions of the tensor-core kernels'
merges and write-backs (``mps2_gb300/csrc/exact_convert.cuh``), compiled
for the host and checked against the C library's conversions: round to
nearest even and truncation to int64, int64 times 2^e to double (against
ldexp of the converted value), and float to double (every 97th bit
pattern)."""
import os
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "exact_convert_test.cpp")


def test_exact_conversions_match_the_c_library(tmp_path):
    exe = str(tmp_path / "exact_convert_test")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", SRC, "-o", exe],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "scale 0" in r.stdout and "f2d 0" in r.stdout, r.stdout

"""The density kernel's fixed-point terms (fdps_sph_gb300/csrc/sph_fixpoint.cuh: FP32 and 32-bit
integer additions in place of a 64-bit float-to-integer conversion) against the C library's
round-half-to-even of t * 2^40: every float t in [0, 16], and seeded sums of 256 terms; the same
header compiled for the host."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_fix40_split_matches_round_half_even(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "fixpoint_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "fdps_sph_gb300", "csrc"), "-o", exe,
                    os.path.join(ROOT, "tests", "cpp", "fixpoint_check.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0" in r.stdout and "checked 1167081319" in r.stdout

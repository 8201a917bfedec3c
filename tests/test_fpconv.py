"""The integer binary64 <-> binary32 conversions of the per-line set-up
kernels (clblm_gb300/csrc/clblm_fpconv.cuh) equal the compiler's conversions
bit for bit: tests/c/fpconv_check.cpp, compiled for the host from the same
header, runs 28 M values (random, ties, round-ups to a power of two, random
bit patterns with subnormals and specials)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def test_fpconv_matches_hardware_conversions(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "fpconv_check"
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", str(ROOT / "clblm_gb300" / "csrc"),
                    str(ROOT / "tests" / "c" / "fpconv_check.cpp"), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "mismatches 0" in r.stdout

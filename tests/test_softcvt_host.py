"""The integer float <-> double conversions of the MPI program's double
chains (geophysics_gb300/csrc/softcvt.cuh), built for the host and checked
against the host's IEEE 754 conversions: every binary32 (widening) and 2^24
binary64 values across underflow, ties and overflow (narrowing).  The GPU
check against the device's own conversions is tests/test_gpu_softcvt.py."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_integer_conversions_match_host_ieee(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "softcvt_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "geophysics_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "softcvt_host_check.cpp"), "-o", exe], check=True)
    out = subprocess.run([exe, str(1 << 24)], check=True, capture_output=True, text=True).stdout.split()
    assert out == ["0", "0"], out

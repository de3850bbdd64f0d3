"""The integer form of the FP32 (hi, lo) position split (rumdeed_gb300/csrc/rd_split.h),
which the position pass, the compaction and the MH proposal packs use, equals the FP64
form hi = (float)v, lo = (float)(v - (double)hi) bit for bit: compiled for the host
with g++ and run on random doubles, rounding ties, carries and the edges of its range."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_split_exact_equals_fp64_form(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "split_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-o", exe, os.path.join(HERE, "split_check.cpp")], check=True)
    r = subprocess.run([exe, "400000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout
    assert "mismatches 0" in r.stdout

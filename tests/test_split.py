"""The integer forms of rumdeed_gb300/csrc/rd_split.h equal the FP64 forms they replace,
bit for bit: the FP32 (hi, lo) position split that the position pass, the compaction and
the MH proposal packs use (hi = (float)v, lo = (float)(v - (double)hi)), on random
doubles, rounding ties, carries and the edges of its range; and the sum of M copies of e
(the serial sampler's escape-probability sum), on random magnitudes, ties and small M.
Compiled for the host with g++."""
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
    assert "mismatches 0 repeat-sums" in r.stdout and r.stdout.strip().endswith("mismatches 0")

"""The handle's host id containers (hann_gb300/csrc/host_maps.h): the flat
id -> list map and the contiguous store of vectors added before training,
built with the host C++ compiler and run against the standard containers on
random insert / replace / erase / lookup / clear sequences (int64 extremes,
re-inserts after erasure, compaction of erased slots)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "..", "hann_gb300", "csrc")


def test_host_maps_against_std(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "host_maps_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, os.path.join(HERE, "host_maps_check.cpp"), "-o", exe],
                   check=True)
    out = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stdout + out.stderr
    assert out.stdout.strip() == "ok"

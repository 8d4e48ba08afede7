"""Staged uploads (nomad_gb300/csrc/host_stage.cpp), the path every rating array of the
caller takes to the device: compiled with g++ against the stand-in runtime of
tests/stub/cuda_runtime.h, whose copies complete late on a thread of their own, and run by
tests/stage_check.cpp over random sets of arrays.  No GPU."""
import os
import shutil
import subprocess

import pytest


def test_staged_uploads_concatenate_exactly(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    here = os.path.dirname(os.path.abspath(__file__))
    root = os.path.dirname(here)
    exe = str(tmp_path / "stage_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-I" + os.path.join(here, "stub"),
                    "-I" + os.path.join(root, "include"), "-I" + os.path.join(root, "nomad_gb300", "csrc"),
                    "-o", exe, os.path.join(here, "stage_check.cpp"),
                    os.path.join(root, "nomad_gb300", "csrc", "host_stage.cpp")], check=True, timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "stage ok" in r.stdout

"""Host-side layout invariants, on the CPU: the CSC build and the route layout of the
asynchronous kernel (row blocks, visit lists, priority groups, grouped routes, initial
queues) and the DSGD / DSGD++ blocks, checked by tests/layout_check.cpp against the
definitions, for several worker counts, thread counts and both row-block balances, with and
without the row counts that the CSC build hands to the layout."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(ROOT, "nomad_gb300", "csrc")


def test_layout_invariants(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "layout_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-pthread", "-I" + os.path.join(ROOT, "include"), "-I" + CSRC,
                    "-o", exe, os.path.join(HERE, "layout_check.cpp"), os.path.join(CSRC, "host_layout.cpp"),
                    os.path.join(CSRC, "host_io.cpp")], check=True, timeout=300)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "layout ok" in r.stdout

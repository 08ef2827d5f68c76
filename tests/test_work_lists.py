"""CPU checks of the step kernels' work lists: the host list builder
(fwi_gb300/csrc/fwi_lists.cpp, no CUDA dependency) compiled with g++ together
with tests/lists_check.cpp and run over ~900 grid shapes (acc 3/4, CPML widths
1..54, narrow and wide grids): single-step coverage, two-step ownership, halo
plainness, read bounds, core tiles, sorted source/receiver lists; the
time-loop planner (two-step passes and single steps) on 3000 random loops; and
the race-freedom of the two-step pipeline's concurrent kernels (read and
write sets of three passes against the dependency graph of two_step_run)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_work_lists(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "lists_check")
    csrc = os.path.join(ROOT, "fwi_gb300", "csrc")
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", csrc, os.path.join(ROOT, "tests", "lists_check.cpp"),
                    os.path.join(csrc, "fwi_lists.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "all ok" in r.stdout

"""The integer emulation of (float)((double)a +- F) used by the kernels
(boids_softfp.h) against the host's double arithmetic."""
import os
import subprocess

import pytest

from conftest import ROOT


def test_soft_double_add_matches_hardware(tmp_path):
    exe = str(tmp_path / "softfp_check")
    subprocess.run(["g++", "-O2", "-std=c++17", "-ffp-contract=off",
                    "-I" + os.path.join(ROOT, "boidssimulatormpi_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "native", "softfp_check.cpp"), "-o", exe],
                   check=True)
    r = subprocess.run([exe, "300000"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in " " + r.stdout

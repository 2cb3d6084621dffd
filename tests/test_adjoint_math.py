"""The adjoint building blocks of the differentiable rollout, on the CPU.

tests/adjoint_check.cpp compiles chipmunk2d_gb300/csrc/cpg_adjoint.cuh (and
the device narrow phase, cpg_narrow.cuh) as host code and checks them
against central finite differences: the reverse of one impulse application,
of the warm start and of the pre-step of a contact, and the dual-number
contact geometry of every shape pair, whose values must equal the narrow
phase's bit for bit.
"""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_adjoint_building_blocks_match_finite_differences(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "adjoint_check")
    subprocess.check_call([gxx, "-std=c++17", "-O2", "-ffp-contract=off",
                           "-I", os.path.join(REPO, "chipmunk2d_gb300", "csrc"),
                           os.path.join(REPO, "tests", "adjoint_check.cpp"), "-o", exe])
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
    assert "0 value mismatches" in r.stdout

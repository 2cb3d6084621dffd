"""The solver's integer clamps, on the CPU.

tests/solver_math_check.cpp compiles chipmunk2d_gb300/csrc/cpg_math.cuh as
host code and checks that dmax0, dclamp_sym and dgt_bits return, bit for
bit, what the reference's cpfmax / cpfclamp compares return
(chipmunk_types.h:137-168), over special values, random bit patterns and
random impulses.  The device solver uses them in place of FP64 compares.
"""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_integer_clamps_match_the_compares(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "solver_math_check")
    subprocess.check_call([gxx, "-std=c++17", "-O2", "-ffp-contract=off",
                           "-I", os.path.join(REPO, "chipmunk2d_gb300", "csrc"),
                           os.path.join(REPO, "tests", "solver_math_check.cpp"), "-o", exe])
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
    assert " 0 mismatches" in r.stdout

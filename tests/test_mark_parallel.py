"""The tree's parallel marking, on the CPU.

tests/mark_check.cpp compiles chipmunk2d_gb300/csrc/cpg_mark.cuh and the
device tree (cpg_tree.cuh) as host code.  Worlds of moving boxes and static
walls are stepped in two copies of the tree: one re-indexes and marks in the
reference's serial order (cpBBTree.c:498-654), the other reinserts the moved
leaves keeping their pairs and runs the parallel marking phases as plain
loops.  Candidates, every leaf's pair list (in order) and the nodes must be
identical after every step.
"""
import os
import shutil
import subprocess

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_parallel_marking_matches_serial_marking(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "mark_check")
    subprocess.check_call([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-frounding-math",
                           "-I", os.path.join(REPO, "chipmunk2d_gb300", "csrc"),
                           os.path.join(REPO, "tests", "mark_check.cpp"), "-o", exe])
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
    assert " 0 mismatches" in r.stdout


def test_tree_box_brackets_decide_exactly(tmp_path):
    """The tree's float brackets (cpg_tree.cuh): every comparison, merge and
    insertion-cost decision they settle must be the one the doubles give,
    on random boxes, near-ties, signed zeros and large magnitudes."""
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no C++ compiler")
    exe = str(tmp_path / "tree_bracket_check")
    subprocess.check_call([gxx, "-std=c++17", "-O2", "-ffp-contract=off", "-frounding-math",
                           "-I", os.path.join(REPO, "chipmunk2d_gb300", "csrc"),
                           os.path.join(REPO, "tests", "tree_bracket_check.cpp"), "-o", exe])
    r = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout
    assert " 0 wrong" in r.stdout

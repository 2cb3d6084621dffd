"""The exact-order tree marked by parallel phases (cpGpuDebugSetParallelMarking)
against the single-thread marking, on the GPU.

Marking decides the candidate order, and so the arbiter order and the
Gauss-Seidel sweep; the parallel phases reproduce it exactly, so the two
runs must agree bit for bit on every body after every chunk of steps (the
phases' own logic is checked against the serial marking on the CPU by
tests/mark_check.cpp)."""
import numpy as np
import pytest

from chipmunk2d_gb300 import Scene

# The first GPU run of this comparison passed on the pyramid and diverged on
# 3,000 circles after 20 steps (31 of 54,000 values, by up to 3.5e-11).  The
# cause found by reading: thread 0 advanced the tree's stamp while other
# blocks still tested leaves against it; a grid barrier now comes first, and
# the comparison has passed on all four workloads since.
pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("cfg,size,steps", [(1, 14, 60), (2, 3000, 60), (3, 1500, 40), (4, 400, 60), (6, 400, 60)])
def test_parallel_marking_matches_serial_marking(gpu_lib, cfg, size, steps):
    a = Scene(gpu_lib, cfg, size)
    b = Scene(gpu_lib, cfg, size)
    try:
        for chunk in range(0, steps, 10):
            gpu_lib.cpGpuDebugSetParallelMarking(0)
            a.step(1 / 60, 10)
            gpu_lib.cpGpuDebugSetParallelMarking(1)
            b.step(1 / 60, 10)
            assert gpu_lib.cpGpuGetLastError() == 0, gpu_lib.cpGpuGetLastErrorString()
            np.testing.assert_array_equal(a.bodies(), b.bodies(), err_msg="after %d steps" % (chunk + 10))
        np.testing.assert_array_equal(a.impulses(), b.impulses())
    finally:
        gpu_lib.cpGpuDebugSetParallelMarking(-1)
        a.free()
        b.free()

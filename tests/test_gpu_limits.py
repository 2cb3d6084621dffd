"""Bounded device waits and table capacities, made to run out on purpose.

Every wait in the device code is bounded, and every table checks its
capacity; running out latches an error bit that the host reports through
cpGpuGetLastError().  These tests make each limit trip -- the coloured
sweep's dataflow waits (a test mode in which no completion is published,
so every wait with a predecessor runs out), the pair cache, the arbiter
table and the tree's node pool (capacities set far too small) -- and check
the reported error, then that the library still steps a fresh space in
parity with the oracle, i.e. the GPU context is intact.  A NaN body state
is stepped as well: the step must finish and the library keep working."""
import numpy as np
import pytest

from chipmunk2d_gb300 import Scene, cpVect

pytestmark = pytest.mark.gpu

CP_GPU_ERR_OVERFLOW = 2
CP_GPU_ERR_TIMEOUT = 4


def still_in_parity(gpu_lib, oracle_lib):
    """A fresh 30-step pyramid on the GPU still matches the oracle."""
    g, o = Scene(gpu_lib, 1, 10), Scene(oracle_lib, 1, 10)
    try:
        for _ in range(30):
            g.step(1 / 60)
            o.step(1 / 60)
        assert gpu_lib.cpGpuGetLastError() == 0, gpu_lib.cpGpuGetLastErrorString()
        b, ob = g.bodies(), o.bodies()
        scale = np.maximum(np.abs(ob).max(axis=0), 1.0)
        assert float((np.abs(b - ob) / scale).max()) <= 1e-12
    finally:
        g.free()
        o.free()


def run_until_error(gpu_lib, sc, steps):
    gpu_lib.cpGpuGetLastError()
    err = 0
    for _ in range(steps):
        sc.step(1 / 60)
        gpu_lib.cpGpuSpaceSync(sc.space)
        err = gpu_lib.cpGpuGetLastError()
        if err:
            break
    return err


def test_dataflow_wait_runs_out_and_reports_a_timeout(gpu_lib, oracle_lib):
    gpu_lib.cpGpuDebugSetFlowSolve(1)
    gpu_lib.cpGpuDebugSetFlowWaitLimit(4096, 1)
    sc = Scene(gpu_lib, 2, 3000)
    try:
        gpu_lib.cpGpuSetSolverMode(sc.space, 1)
        err = run_until_error(gpu_lib, sc, 40)
    finally:
        gpu_lib.cpGpuDebugSetFlowWaitLimit(0, 0)
        gpu_lib.cpGpuDebugSetFlowSolve(0)
        sc.free()
    assert err == CP_GPU_ERR_TIMEOUT, err
    still_in_parity(gpu_lib, oracle_lib)


@pytest.mark.parametrize("caps", [(1, 0, 0, 0), (0, -1, 4, 0), (0, -1, 0, 40)],
                         ids=["pairs", "arbiters", "nodes"])
def test_table_overflow_is_latched_and_reported(gpu_lib, oracle_lib, caps):
    gpu_lib.cpGpuDebugSetCapacities(*caps)
    sc = Scene(gpu_lib, 4, 300)
    try:
        err = run_until_error(gpu_lib, sc, 90)
    finally:
        gpu_lib.cpGpuDebugSetCapacities(0, -1, 0, 0)
        sc.free()
    assert err == CP_GPU_ERR_OVERFLOW, err
    still_in_parity(gpu_lib, oracle_lib)


def test_nan_body_state_is_stepped_without_a_fault(gpu_lib, oracle_lib):
    """One body of a pyramid gets a NaN velocity.  The step must finish on
    the device without a fault and the library must keep working.  (Results
    are not compared: the reference's IEEE min and max carry a NaN box up
    its tree and every query through it fails, while the device tree's
    integer comparisons order NaN above every number.)"""
    gpu_lib.cpGpuGetLastError()
    g = Scene(gpu_lib, 1, 10)
    try:
        b = gpu_lib.cpBodyNew(1.0, 100.0)
        gpu_lib.cpSpaceAddBody(g.space, b)
        gpu_lib.cpBodySetPosition(b, cpVect(0.0, 50.0))
        gpu_lib.cpSpaceAddShape(g.space, gpu_lib.cpCircleShapeNew(b, 2.0, cpVect(0.0, 0.0)))
        gpu_lib.cpBodySetVelocity(b, cpVect(float("nan"), 0.0))
        for _ in range(20):
            g.step(1 / 60)
        gpu_lib.cpGpuSpaceSync(g.space)
        assert gpu_lib.cpGpuGetLastError() in (0, CP_GPU_ERR_OVERFLOW)
        assert np.isnan(g.bodies()[-1, 2])
    finally:
        g.free()
    still_in_parity(gpu_lib, oracle_lib)

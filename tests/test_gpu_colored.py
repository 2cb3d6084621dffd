"""Coloured solver mode (CP_GPU_SOLVER_COLORED): sweep-and-prune broadphase
and graph-coloured Gauss-Seidel.

* The broadphase pair set must equal the reference tree's: the pairs whose
  boxes intersect, compared as sets of (min, max) shape ids, from identical
  body states (the oracle's state is copied in before every step).
* The coloured sweep changes the Gauss-Seidel order, so its trajectories
  differ from the reference's; it is judged by solver quality instead: the
  velocity residual after each iteration and the largest penetration,
  against the reference-order sweep from the same state.
* Units of one colour share no body, so the result does not depend on the
  order inside a colour: two runs are bit-identical.
"""
import numpy as np
import pytest

from chipmunk2d_gb300 import Scene

pytestmark = pytest.mark.gpu


def colored(lib, cfg, size, seed=None):
    sc = Scene(lib, cfg, size, seed=seed)
    lib.cpGpuSetSolverMode(sc.space, 1)
    return sc


@pytest.mark.parametrize("cfg,size,steps", [(2, 3000, 25), (3, 1500, 20), (4, 400, 25), (1, 14, 10)])
def test_sweep_and_prune_pair_set_matches_tree(gpu_lib, oracle_lib, cfg, size, steps):
    g = colored(gpu_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    try:
        for s in range(steps):
            g.set_bodies(o.bodies())
            g.step(1 / 60)
            o.step(1 / 60)
            assert gpu_lib.cpGpuGetLastError() == 0, gpu_lib.cpGpuGetLastErrorString()
            pg, po = g.candidates(), o.candidates()
            assert pg == po, "step %d: %d GPU pairs vs %d tree pairs; %d missing, %d extra" % (
                s, len(pg), len(po), len(po - pg), len(pg - po))
    finally:
        g.free()
        o.free()


def solver_quality(lib, sc, mode, iters, dt=1 / 60):
    out = np.zeros(3 * iters)
    assert lib.cpGpuSolverQuality(sc.space, mode, dt, iters, out.ctypes.data) == 0, lib.cpGpuGetLastErrorString()
    return out.reshape(iters, 3)


@pytest.mark.parametrize("cfg,size,steps", [(2, 3000, 240), (3, 1500, 150)], ids=["circles", "mixed"])
def test_colored_contact_quality_matches_reference_order(gpu_lib, oracle_lib, cfg, size, steps):
    """From one state (a pile after `steps` reference-order steps), the next
    step is solved in both modes with 1 .. N iterations (cpGpuSolverQuality).
    The coloured sweep is judged against the reference-order sweep by the
    per-iteration velocity residual (normal complementarity and friction
    cone, RMS over contacts) and by the largest penetration after the next
    position update: after the last iteration, its residuals within twice
    the reference order's (plus 1% of the first iteration's, for residuals
    near zero) and its penetration within 5% of it (plus 1e-3); and both
    sweeps must converge: the last iteration's normal residual below half
    the first's."""
    g = Scene(gpu_lib, cfg, size)
    try:
        g.step(1 / 60, steps)
        assert gpu_lib.cpGpuGetLastError() == 0
        iters = gpu_lib.cpSpaceGetIterations(g.space)
        before = g.bodies()
        qo = solver_quality(gpu_lib, g, 0, iters)
        qc = solver_quality(gpu_lib, g, 1, iters)
        np.testing.assert_array_equal(g.bodies(), before)      # the space is left as it was
        for k in range(iters):
            print("iteration %2d  ordered: normal %.3e friction %.3e pen %.4f   coloured: normal %.3e friction %.3e pen %.4f"
                  % (k + 1, *qo[k], *qc[k]))
        assert qo[-1, 0] < 0.5 * qo[0, 0] and qc[-1, 0] < 0.5 * qc[0, 0]
        for j in (0, 1):
            assert qc[-1, j] <= 2.0 * qo[-1, j] + 0.01 * qo[0, j], (j, qc[-1], qo[-1])
        assert qc[-1, 2] <= 1.05 * qo[-1, 2] + 1e-3, (qc[-1, 2], qo[-1, 2])
    finally:
        g.free()


def test_colored_runs_are_deterministic(gpu_lib):
    a = colored(gpu_lib, 2, 2000)
    b = colored(gpu_lib, 2, 2000)
    try:
        a.step(1 / 60, 60)
        b.step(1 / 60, 60)
        np.testing.assert_array_equal(a.bodies(), b.bodies())
    finally:
        a.free()
        b.free()


def test_solver_mode_rejects_unknown_values(gpu_lib):
    sc = Scene(gpu_lib, 1, 14)
    try:
        gpu_lib.cpGpuGetLastError()
        gpu_lib.cpGpuSetSolverMode(sc.space, 7)
        assert gpu_lib.cpGpuGetLastError() == 6
        assert gpu_lib.cpGpuGetSolverMode(sc.space) == 0
    finally:
        sc.free()


def test_colour_reuse_stays_deterministic_across_recolouring(gpu_lib):
    """Units that were units of the previous step keep their colour; every
    64th step colours all units afresh.  A unit kept with a colour another
    unit of its body also holds would race in the solve, so bit-identical
    runs over both kinds of step show the colouring stays proper."""
    a = colored(gpu_lib, 2, 20000)
    b = colored(gpu_lib, 2, 20000)
    try:
        for chunk in range(3):
            a.step(1 / 60, 50)
            b.step(1 / 60, 50)
            assert gpu_lib.cpGpuGetLastError() == 0, gpu_lib.cpGpuGetLastErrorString()
            np.testing.assert_array_equal(a.bodies(), b.bodies(), err_msg="after %d steps" % (50 * chunk + 50))
    finally:
        a.free()
        b.free()


def test_colour_count_with_reuse_stays_near_fresh_colouring(gpu_lib):
    sc = colored(gpu_lib, 2, 20000)
    stats = np.zeros(8, dtype=np.int32)
    try:
        sc.step(1 / 60, 128)          # the 128th step colours afresh
        gpu_lib.cpGpuGetStepStats(sc.space, stats.ctypes.data, 8)
        fresh = int(stats[6])
        worst = 0
        for _ in range(40):
            sc.step(1 / 60)
            gpu_lib.cpGpuGetStepStats(sc.space, stats.ctypes.data, 8)
            worst = max(worst, int(stats[6]))
        assert gpu_lib.cpGpuGetLastError() == 0
        assert 2 <= fresh <= 16, fresh
        assert worst <= fresh + 3, (fresh, worst)
    finally:
        sc.free()


@pytest.mark.parametrize("cfg,size,steps", [(2, 20000, 130), (3, 3000, 60)])
def test_dataflow_sweep_matches_barrier_sweep(gpu_lib, cfg, size, steps):
    """The coloured sweep by dataflow (each unit waits for the units before
    it on its bodies) applies every body's updates in the same order as the
    sweep with a grid barrier after each colour: bit-identical results, on
    circles across a recolouring step and on mixed shapes with joints."""
    a = colored(gpu_lib, cfg, size)
    b = colored(gpu_lib, cfg, size)
    try:
        for chunk in range(0, steps, 10):
            gpu_lib.cpGpuDebugSetFlowSolve(1)
            a.step(1 / 60, 10)
            gpu_lib.cpGpuDebugSetFlowSolve(0)
            b.step(1 / 60, 10)
            assert gpu_lib.cpGpuGetLastError() == 0, gpu_lib.cpGpuGetLastErrorString()
            np.testing.assert_array_equal(a.bodies(), b.bodies(), err_msg="after %d steps" % (chunk + 10))
        # per-body sums of the arbiters' impulses follow the solve list,
        # whose order inside a colour is not fixed: equal up to rounding
        np.testing.assert_allclose(a.impulses(), b.impulses(), rtol=1e-12, atol=1e-12)
    finally:
        gpu_lib.cpGpuDebugSetFlowSolve(0)
        a.free()
        b.free()


@pytest.mark.parametrize("cfg,size,steps,flow", [(2, 20000, 130, 0), (3, 3000, 60, 0), (3, 3000, 30, 1)])
def test_warm_start_gather_matches_sweep(gpu_lib, cfg, size, steps, flow):
    """The coloured mode's warm start as a per-body gather of the cached
    impulses in colour order gives every body the same updates in the same
    order as the sweep's first pass: bit-identical results, with joints
    (mixed scene) and under the dataflow sweep too."""
    a = colored(gpu_lib, cfg, size)
    b = colored(gpu_lib, cfg, size)
    gpu_lib.cpGpuDebugSetFlowSolve(flow)
    try:
        for chunk in range(0, steps, 10):
            gpu_lib.cpGpuDebugSetWarmStartGather(1)
            a.step(1 / 60, 10)
            gpu_lib.cpGpuDebugSetWarmStartGather(0)
            b.step(1 / 60, 10)
            assert gpu_lib.cpGpuGetLastError() == 0, gpu_lib.cpGpuGetLastErrorString()
            np.testing.assert_array_equal(a.bodies(), b.bodies(), err_msg="after %d steps" % (chunk + 10))
    finally:
        gpu_lib.cpGpuDebugSetWarmStartGather(0)
        gpu_lib.cpGpuDebugSetFlowSolve(0)
        a.free()
        b.free()

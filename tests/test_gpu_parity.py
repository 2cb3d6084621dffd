"""GPU parity: libchipmunk_gb300 (reference-order solver) against the CPU
oracle, through the C ABI, on the seeded workloads.

Tolerance: 1e-12 relative per step, per state component, scaled by the
component's magnitude over all bodies (max(|x|, 1)).  The device and the
host round every +,-,*,/,sqrt identically (no FMA contraction on either
side); the remaining source of difference is the last bit of sin/cos in
the body transforms, which this tolerance covers.

"Teacher-forced" runs copy the oracle's complete state into the GPU before
every step -- the bodies and the warm-start impulses the step begins from
(every arbiter of the last solve list and every joint) -- so each
comparison measures one step from identical inputs; "free" runs compare two
independent rollouts.  Arbiter lists (shape pairs, contact counts, solve
order) must match exactly.
"""
import numpy as np
import pytest

from chipmunk2d_gb300 import Scene
import known_answers as ka

pytestmark = pytest.mark.gpu

RTOL = 1e-12
# Bias velocities (v_bias, w_bias: the position-correction pseudo-velocity
# a step leaves for the next position update) carry the contact normals'
# conditioning: a 2 cm polygon edge at 60 units from the origin turns the
# one-ulp sin/cos difference of a body's rotation into one ulp of 60 in its
# world vertices and 3e-13 in that edge's normal (measured on the joints
# workload, where positions, velocities and impulses stayed within 3e-14).
# They are held to 1e-11; every other component to RTOL.
BIAS_COLS = [9, 10, 11]
RTOL_BIAS = 1e-11


def rel_err(a, b):
    """Largest component error, each column scaled by max(|b|, 1)."""
    if a.size == 0 and b.size == 0:
        return 0.0
    scale = np.maximum(np.abs(b).max(axis=0), 1.0)
    return float((np.abs(a - b) / scale).max())


def check_gpu_error(lib):
    e = lib.cpGpuGetLastError()
    assert e == 0, lib.cpGpuGetLastErrorString().decode()


def force(g, o):
    """The oracle's state into the GPU space: bodies, then the accumulated
    impulses of the arbiters and joints (same solve list on both sides)."""
    g.set_bodies(o.bodies())
    assert g.set_impulses(o.arbiters(), o.constraints()) == 0


def compare_step(g, o, step, bias_tol=RTOL_BIAS):
    gb, ob = g.bodies(), o.bodies()
    ga, oa = g.arbiters(), o.arbiters()
    assert ga.shape == oa.shape, "step %d: %d arbiters on the GPU, %d in the oracle" % (step, len(ga), len(oa))
    np.testing.assert_array_equal(ga[:, :3], oa[:, :3], err_msg="step %d: arbiter pairs/counts/order" % step)
    if len(ob):
        eb_bias = rel_err(gb[:, BIAS_COLS], ob[:, BIAS_COLS])
        assert eb_bias <= bias_tol, "step %d: bias velocities differ by %.3g" % (step, eb_bias)
        keep = [c for c in range(gb.shape[1]) if c not in BIAS_COLS]
        gb, ob = gb[:, keep], ob[:, keep]
    eb = rel_err(gb, ob)
    ea = rel_err(ga[:, 4:], oa[:, 4:])
    gj, oj = g.constraints(), o.constraints()
    ej = rel_err(gj, oj) if len(oj) else 0.0
    return eb, ea, ej


CASES = [
    ("pyramid", 1, 14, 1 / 60, 300),
    ("circles", 2, 1500, 1 / 60, 120),
    ("mixed", 3, 1200, 1 / 60, 80),
    ("tumble", 4, 300, 1 / 60, 120),
    ("adjoint", 5, 64, 1 / 120, 120),
    ("joints", 6, 200, 1 / 60, 200),
    ("machines", 7, 40, 1 / 60, 300),
]


@pytest.mark.parametrize("name,cfg,size,dt,steps", CASES, ids=[c[0] for c in CASES])
def test_teacher_forced_per_step(gpu_lib, oracle_lib, name, cfg, size, dt, steps):
    g = Scene(gpu_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    worst = [0.0, 0.0, 0.0]
    try:
        for s in range(steps):
            force(g, o)
            g.step(dt)
            o.step(dt)
            check_gpu_error(gpu_lib)
            errs = compare_step(g, o, s)
            worst = [max(a, b) for a, b in zip(worst, errs)]
            assert max(errs) <= RTOL, "step %d: body %.3g arbiter %.3g joint %.3g" % ((s,) + errs)
    finally:
        g.free()
        o.free()
    print("%s: worst rel err bodies %.3g arbiters %.3g joints %.3g" % (name, *worst))


@pytest.mark.parametrize("cfg,size", [(6, 200), (3, 600), (1, 14), (4, 150)], ids=["joints", "mixed", "pyramid", "tumble"])
def test_teacher_forced_with_objects_added_and_removed(gpu_lib, oracle_lib, cfg, size):
    """Objects added and removed between steps (cpx_scene_edit every 10
    steps: removals, additions, constraint churn, body-type changes).  The
    GPU rebuilds its set at the next step, carrying the tree and arbiter
    cache over, and must stay on the oracle's per-step results: same
    arbiter lists, bodies and joints within the per-step bounds.  On an
    edit step only the bodies are forced (the arbiter lists of the two
    sides are compared after the step)."""
    g = Scene(gpu_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    worst = 0.0
    try:
        for s in range(150):
            edited = (s % 10 == 5)
            if edited:
                assert g.edit(s // 10, 7) == o.edit(s // 10, 7)
                g.set_bodies(o.bodies())
            else:
                force(g, o)
            g.step(1 / 60)
            o.step(1 / 60)
            check_gpu_error(gpu_lib)
            assert g.bodies().shape == o.bodies().shape
            errs = compare_step(g, o, s)
            worst = max(worst, *errs)
            assert max(errs) <= RTOL, "step %d: body %.3g arbiter %.3g joint %.3g" % ((s,) + errs)
    finally:
        g.free()
        o.free()
    print("edits, workload %d: worst rel err %.3g" % (cfg, worst))


FREE_RUN_DRIFT = 1e-9


@pytest.mark.parametrize("name,cfg,size,dt,steps", [CASES[0], CASES[1], CASES[2], CASES[5], CASES[6]],
                         ids=["pyramid", "circles", "mixed", "joints", "machines"])
def test_teacher_forced_whole_grid_solve(gpu_lib, oracle_lib, name, cfg, size, dt, steps):
    """The whole-grid solve (four lanes per contact, a grid barrier between
    levels), which large single worlds use, against the oracle."""
    gpu_lib.cpGpuDebugSetWholeGridSolve(1)
    try:
        g = Scene(gpu_lib, cfg, size)
        o = Scene(oracle_lib, cfg, size)
        try:
            worst = 0.0
            for s in range(min(steps, 60)):
                force(g, o)
                g.step(dt)
                o.step(dt)
                check_gpu_error(gpu_lib)
                worst = max(worst, *compare_step(g, o, s))
            assert worst <= RTOL, worst
        finally:
            g.free()
            o.free()
    finally:
        gpu_lib.cpGpuDebugSetWholeGridSolve(0)


def test_pyramid_free_run_1000_steps(gpu_lib, oracle_lib):
    """The full 1000-step pyramid rollout as two independent runs.  The
    per-step contract (1e-12, teacher-forced tests above) holds; over a free
    run, last-bit differences between the device's and the host C library's
    sin/cos compound, so this bounds the accumulated drift instead.  The
    arbiter lists must still agree exactly at every checkpoint."""
    g = Scene(gpu_lib, 1, 14)
    o = Scene(oracle_lib, 1, 14)
    try:
        worst = 0.0
        for s in range(1000):
            g.step(1 / 60)
            o.step(1 / 60)
            if s % 50 == 49 or s < 5:
                check_gpu_error(gpu_lib)
                eb, ea, _ = compare_step(g, o, s, bias_tol=FREE_RUN_DRIFT)
                worst = max(worst, eb, ea)
        print("pyramid free-run drift after 1000 steps: %.3g" % worst)
        assert worst <= FREE_RUN_DRIFT, worst
        np.testing.assert_allclose(g.impulses(), o.impulses(), rtol=0, atol=1e-7)
    finally:
        g.free()
        o.free()


def test_known_answer_time_stepping(gpu_lib):
    assert ka.time_stepping(gpu_lib) == ka.TIME_STEPPING_EXPECTED


def test_known_answer_resting_ball(gpu_lib):
    y, slop = ka.resting_ball(gpu_lib)
    assert abs(y - 2.0) <= 1.1 * slop


@pytest.mark.parametrize("case", range(len(ka.HULL_CASES)))
def test_known_answer_convex_hull(gpu_lib, case):
    pts, count, expected = ka.HULL_CASES[case]
    ka.check_hull_case(gpu_lib, pts, count, expected)


def test_public_getters_and_impulses_match(gpu_lib, oracle_lib):
    g = Scene(gpu_lib, 4, 200)
    o = Scene(oracle_lib, 4, 200)
    try:
        for s in range(60):
            force(g, o)
            g.step(1 / 60)
            o.step(1 / 60)
        check_gpu_error(gpu_lib)
        assert rel_err(g.public(), o.public()) <= RTOL
        assert rel_err(g.impulses(), o.impulses()) <= 1e-10
    finally:
        g.free()
        o.free()


@pytest.mark.parametrize("cfg", [4, 6, 7], ids=["tumble", "joints", "machines"])
def test_batched_worlds_match_single_worlds(gpu_lib, oracle_lib, cfg):
    """Uneven worlds stepped together in one batch match the oracle stepping
    each world alone: tumble worlds, and worlds of pin and slide joints with
    filtered shapes."""
    import ctypes
    sizes = (ctypes.c_int * 24)()
    gpu_lib.cpx_batch_sizes(24, 3, ctypes.cast(sizes, ctypes.c_void_p))
    if cfg == 6:
        sizes = [40 + (sizes[i] * 160) // 512 for i in range(24)]
    elif cfg == 7:
        sizes = [2 + (sizes[i] * 30) // 512 for i in range(24)]
    gs = [Scene(gpu_lib, cfg, sizes[i], seed=100 + i) for i in range(24)]
    os_ = [Scene(oracle_lib, cfg, sizes[i], seed=100 + i) for i in range(24)]
    batch = gpu_lib.cpGpuBatchNew()
    try:
        for g in gs:
            assert gpu_lib.cpGpuBatchAddSpace(batch, g.space) >= 0
        worst = 0.0
        for s in range(60):
            for g, o in zip(gs, os_):
                force(g, o)
            assert gpu_lib.cpGpuBatchStep(batch, 1 / 60, 1, 0) == 0
            for o in os_:
                o.step(1 / 60)
            check_gpu_error(gpu_lib)
            for g, o in zip(gs, os_):
                eb, ea, _ = compare_step(g, o, s)
                worst = max(worst, eb, ea)
        assert worst <= RTOL, worst
    finally:
        gpu_lib.cpGpuBatchFree(batch)
        for g in gs:
            g.free()
        for o in os_:
            o.free()


def _batch_run(lib, n, steps, use_graph, autotune):
    import ctypes
    sizes = (ctypes.c_int * n)()
    lib.cpx_batch_sizes(n, 3, ctypes.cast(sizes, ctypes.c_void_p))
    gs = [Scene(lib, 4, min(sizes[i], 96), seed=300 + i) for i in range(n)]
    batch = lib.cpGpuBatchNew()
    lib.cpGpuSetAutotune(autotune)
    try:
        for g in gs:
            assert lib.cpGpuBatchAddSpace(batch, g.space) >= 0
        for _ in range(steps // 4):
            assert lib.cpGpuBatchStep(batch, 1 / 60, 4, use_graph) == 0
        check_gpu_error(lib)
        tune = (ctypes.c_int * 2)()
        lib.cpGpuBatchGetTuning(batch, ctypes.cast(tune, ctypes.c_void_p))
        return [g.bodies() for g in gs], (tune[0], tune[1])
    finally:
        lib.cpGpuSetAutotune(1)
        lib.cpGpuBatchFree(batch)
        for g in gs:
            g.free()


def test_graph_replay_and_online_tuning_do_not_change_results(gpu_lib):
    """A many-world batch stepped through its CUDA graph, with the online
    tuner trying launch shapes on the way, ends bit-identical to plain
    launches with the default shapes."""
    # the first tuning window opens at step 32 and takes 12 steps
    base, t0 = _batch_run(gpu_lib, 160, 48, 0, 0)
    graph, t1 = _batch_run(gpu_lib, 160, 48, 1, 1)
    assert t0 == (0, -1)
    assert t1[0] in (64, 128, 256) and t1[1] in (-1, 0)
    for a, b in zip(base, graph):
        np.testing.assert_array_equal(a, b)

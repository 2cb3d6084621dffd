"""Pins the CPU restatement (oracle/cp_oracle.c) to the unmodified reference.

Both libraries are driven through the same C API on the same seeded scenes;
after every step the full simulation state -- every dynamic body, every
arbiter in solve order with all contact fields, every joint -- must be
bit-identical.  Runs where the reference was built (oracle/build_ref.sh);
skipped elsewhere.  The known-answer cases of the reference's own tests run
on both libraries.
"""
import numpy as np
import pytest

from chipmunk2d_gb300 import Scene
import known_answers as ka

# (workload, size, steps, dt): small sizes keep the CPU suite to seconds.
CASES = [
    (1, 14, 400, 1 / 60),
    (2, 800, 200, 1 / 60),
    (3, 900, 120, 1 / 60),
    (4, 300, 200, 1 / 60),
    (5, 64, 240, 1 / 120),
    (6, 200, 300, 1 / 60),
    (7, 40, 400, 1 / 60),
]


@pytest.mark.parametrize("cfg,size,steps,dt", CASES)
def test_oracle_bit_exact_per_step(ref_lib, oracle_lib, cfg, size, steps, dt):
    r = Scene(ref_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    try:
        assert r.nbodies == o.nbodies
        for s in range(steps):
            r.step(dt)
            o.step(dt)
            np.testing.assert_array_equal(o.bodies(), r.bodies(), err_msg="bodies, step %d" % s)
            np.testing.assert_array_equal(o.arbiters(), r.arbiters(), err_msg="arbiters, step %d" % s)
            np.testing.assert_array_equal(o.constraints(), r.constraints(), err_msg="joints, step %d" % s)
        np.testing.assert_array_equal(o.public(), r.public())
        np.testing.assert_array_equal(o.impulses(), r.impulses())
    finally:
        r.free()
        o.free()


@pytest.mark.parametrize("cfg,size", [(6, 120), (4, 150), (3, 300), (1, 14)])
def test_oracle_bit_exact_with_objects_added_and_removed(ref_lib, oracle_lib, cfg, size):
    """Every 10 steps a round of edits between steps (cpx_scene_edit): shapes
    and bodies leave, new ones enter, a constraint leaves and a pin joint
    joins, bodies turn static or kinematic and back.  The state after every
    step must stay bit-identical to the reference's."""
    r = Scene(ref_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    eq = lambda x, y: np.array_equal(x, y, equal_nan=True)
    try:
        for s in range(200):
            if s % 10 == 5:
                assert r.edit(s // 10, 7) == o.edit(s // 10, 7)
            r.step(1 / 60)
            o.step(1 / 60)
            assert eq(o.bodies(), r.bodies()), "bodies, step %d" % s
            assert eq(o.arbiters(), r.arbiters()), "arbiters, step %d" % s
            assert eq(o.constraints(), r.constraints()), "joints, step %d" % s
        assert eq(o.public(), r.public())
    finally:
        r.free()
        o.free()


@pytest.mark.parametrize("which", ["ref", "oracle"])
def test_time_stepping_known_answer(request, which):
    lib = request.getfixturevalue(which + "_lib")
    assert ka.time_stepping(lib) == ka.TIME_STEPPING_EXPECTED


@pytest.mark.parametrize("which", ["ref", "oracle"])
def test_resting_ball_known_answer(request, which):
    lib = request.getfixturevalue(which + "_lib")
    y, slop = ka.resting_ball(lib)
    assert abs(y - 2.0) <= 1.1 * slop


@pytest.mark.parametrize("which", ["ref", "oracle"])
@pytest.mark.parametrize("case", range(len(ka.HULL_CASES)))
def test_convex_hull_known_answer(request, which, case):
    lib = request.getfixturevalue(which + "_lib")
    pts, count, expected = ka.HULL_CASES[case]
    ka.check_hull_case(lib, pts, count, expected)


def test_random_hulls_match_reference(ref_lib, oracle_lib):
    for n, seed in ((100, 1), (1000, 2), (10000, 3)):
        assert ka.random_hull_fixed_point(oracle_lib, n, seed) == ka.random_hull_fixed_point(ref_lib, n, seed)


@pytest.mark.parametrize("cfg,size,steps", [(1, 14, 60), (2, 600, 150), (3, 600, 80), (6, 150, 100), (7, 30, 100)])
def test_oracle_spatial_queries_bit_exact(ref_lib, oracle_lib, cfg, size, steps):
    """Point, nearest-point, segment, first-hit, box and single-shape queries
    (cpSpaceQuery.c, cpShape.c) on the seeded scenes before the first step,
    after some steps and after edits: every callback, in order, and every
    result must be bit-identical to the reference's."""
    r = Scene(ref_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    try:
        np.testing.assert_array_equal(o.queries(1, 140), r.queries(1, 140), err_msg="before the first step")
        for s in range(steps):
            r.step(1 / 60)
            o.step(1 / 60)
        qo, qr = o.queries(2, 700), r.queries(2, 700)
        assert len(qr) > 700
        np.testing.assert_array_equal(qo, qr, err_msg="after %d steps" % steps)
        if cfg in (1, 3, 6):
            assert r.edit(0, 7) == o.edit(0, 7)
            np.testing.assert_array_equal(o.queries(3, 140), r.queries(3, 140), err_msg="after edits")
    finally:
        r.free()
        o.free()

"""Sleeping (src/cpSpaceComponent.c): idle times, the contact graph,
components falling asleep and waking.

On the CPU the oracle is pinned to the reference bit for bit after every
step, with the sleeping flag of every body compared too.  On the GPU each
step is teacher-forced from the oracle (bodies and accumulated impulses)
and compared as in test_gpu_parity.py; the sleeping flags must agree
exactly at every step.  Halfway through, an impulse on a sleeping body
wakes its component on both sides.
"""
import ctypes

import numpy as np
import pytest

from chipmunk2d_gb300 import Scene, cpVect
from test_gpu_parity import check_gpu_error, compare_step, force

# (workload, size, steps): the pyramid falls asleep whole, the chains of the
# joints workload doze in pieces and wake, the machines sleep where their
# motors do not reach, and the mixed pile sleeps here and there.
CASES = [(1, 14, 360), (6, 200, 400), (7, 40, 400), (3, 600, 240)]
IDS = ["pyramid", "joints", "machines", "mixed"]
THRESHOLD = 0.3


def bind_sleep(lib):
    lib.cpSpaceSetSleepTimeThreshold.argtypes = [ctypes.c_void_p, ctypes.c_double]
    lib.cpBodyIsSleeping.argtypes = [ctypes.c_void_p]
    lib.cpBodyIsSleeping.restype = ctypes.c_ubyte
    lib.cpx_scene_body.argtypes = [ctypes.c_void_p, ctypes.c_int]
    lib.cpx_scene_body.restype = ctypes.c_void_p
    lib.cpBodyApplyImpulseAtWorldPoint.argtypes = [ctypes.c_void_p, cpVect, cpVect]
    lib.cpBodyGetPosition.argtypes = [ctypes.c_void_p]
    lib.cpBodyGetPosition.restype = cpVect


def sleeping(sc):
    lib = sc.lib
    return np.array([lib.cpBodyIsSleeping(lib.cpx_scene_body(sc.h, i)) for i in range(sc.nbodies)], dtype=np.uint8)


def wake_one(sc, flags):
    """An upward impulse on the first sleeping body (cpBody.c:550-557 wakes
    its component)."""
    idx = int(np.flatnonzero(flags)[0])
    b = sc.lib.cpx_scene_body(sc.h, idx)
    sc.lib.cpBodyApplyImpulseAtWorldPoint(b, cpVect(0.0, 5.0), sc.lib.cpBodyGetPosition(b))
    return idx


@pytest.mark.parametrize("cfg,size,steps", CASES, ids=IDS)
def test_oracle_bit_exact_with_sleeping(ref_lib, oracle_lib, cfg, size, steps):
    bind_sleep(ref_lib)
    bind_sleep(oracle_lib)
    r = Scene(ref_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    try:
        for sc in (r, o):
            sc.lib.cpSpaceSetSleepTimeThreshold(sc.space, THRESHOLD)
        asleep = 0
        for s in range(steps):
            if s == steps // 2:
                fr = sleeping(r)
                if fr.any():
                    assert wake_one(r, fr) == wake_one(o, sleeping(o))
            r.step(1 / 60)
            o.step(1 / 60)
            fr, fo = sleeping(r), sleeping(o)
            np.testing.assert_array_equal(fo, fr, err_msg="sleeping flags, step %d" % s)
            asleep = max(asleep, int(fr.sum()))
            np.testing.assert_array_equal(o.bodies(), r.bodies(), err_msg="bodies, step %d" % s)
            np.testing.assert_array_equal(o.arbiters(), r.arbiters(), err_msg="arbiters, step %d" % s)
            np.testing.assert_array_equal(o.constraints(), r.constraints(), err_msg="joints, step %d" % s)
        assert asleep > 0
        np.testing.assert_array_equal(o.public(), r.public())
    finally:
        r.free()
        o.free()


@pytest.mark.gpu
@pytest.mark.parametrize("cfg,size,steps", CASES, ids=IDS)
def test_teacher_forced_with_sleeping(gpu_lib, oracle_lib, cfg, size, steps):
    bind_sleep(gpu_lib)
    bind_sleep(oracle_lib)
    g = Scene(gpu_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    try:
        for sc in (g, o):
            sc.lib.cpSpaceSetSleepTimeThreshold(sc.space, THRESHOLD)
        fell = rose = 0
        prev = sleeping(o)
        worst = 0.0
        for s in range(steps):
            if s == steps // 2 and prev.any():
                assert wake_one(o, prev) == wake_one(g, sleeping(g))
            if s > 0:
                force(g, o)
            g.step(1 / 60)
            o.step(1 / 60)
            check_gpu_error(gpu_lib)
            fg, fo = sleeping(g), sleeping(o)
            np.testing.assert_array_equal(fg, fo, err_msg="sleeping flags, step %d" % s)
            fell += int(np.sum(fo & ~prev))
            rose += int(np.sum(prev & ~fo))
            prev = fo
            eb, ea, _ = compare_step(g, o, s)
            worst = max(worst, eb, ea)
        print("workload %d with sleeping: %d bodies fell asleep, %d woke; worst rel err %.3g" % (cfg, fell, rose, worst))
        assert fell > 0
        np.testing.assert_allclose(g.public(), o.public(), rtol=1e-9, atol=1e-9)
    finally:
        g.free()
        o.free()

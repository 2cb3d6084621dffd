"""Collision handlers (cpSpace.c:378-413, cpSpaceStep.c:235-325, 439-444)
on seeded workloads, with the callbacks written in Python.

Every shape gets a collision type from its index; three handlers and a
wildcard count their calls, refuse every third first touch of one type
pair (begin returns false), halve the friction of another in pre-solve and
ignore some of its contacts, and sum the solved impulses in post-solve.
On the CPU the oracle is pinned to the reference bit for bit after every
step, callback counts included; on the GPU each step is teacher-forced
from the oracle and compared as in test_gpu_parity.py, with the callback
counts exact at every step.
"""
import ctypes

import numpy as np
import pytest

from chipmunk2d_gb300 import Scene, cpVect
from test_gpu_parity import check_gpu_error, compare_step, force

P = ctypes.c_void_p
BEGIN = ctypes.CFUNCTYPE(ctypes.c_ubyte, P, P, P)
PRESOLVE = ctypes.CFUNCTYPE(ctypes.c_ubyte, P, P, P)
POSTSOLVE = ctypes.CFUNCTYPE(None, P, P, P)
SEPARATE = ctypes.CFUNCTYPE(None, P, P, P)
WILDCARD = ctypes.c_size_t(-1).value


class Handler(ctypes.Structure):
    """cpCollisionHandler (cpSpace.h:41-66)."""
    _fields_ = [("typeA", ctypes.c_size_t), ("typeB", ctypes.c_size_t),
                ("beginFunc", BEGIN), ("preSolveFunc", PRESOLVE),
                ("postSolveFunc", POSTSOLVE), ("separateFunc", SEPARATE), ("userData", P)]


def bind(lib):
    lib.cpSpaceAddCollisionHandler.restype = ctypes.POINTER(Handler)
    lib.cpSpaceAddCollisionHandler.argtypes = [P, ctypes.c_size_t, ctypes.c_size_t]
    lib.cpSpaceAddWildcardHandler.restype = ctypes.POINTER(Handler)
    lib.cpSpaceAddWildcardHandler.argtypes = [P, ctypes.c_size_t]
    lib.cpShapeSetCollisionType.argtypes = [P, ctypes.c_size_t]
    lib.cpx_scene_shape.restype = P
    lib.cpx_scene_shape.argtypes = [P, ctypes.c_int]
    lib.cpArbiterGetFriction.restype = ctypes.c_double
    lib.cpArbiterGetFriction.argtypes = [P]
    lib.cpArbiterSetFriction.argtypes = [P, ctypes.c_double]
    lib.cpArbiterGetNormal.restype = cpVect
    lib.cpArbiterGetNormal.argtypes = [P]
    lib.cpArbiterTotalImpulse.restype = cpVect
    lib.cpArbiterTotalImpulse.argtypes = [P]
    lib.cpArbiterIgnore.restype = ctypes.c_ubyte
    lib.cpArbiterIgnore.argtypes = [P]
    lib.cpArbiterIsFirstContact.restype = ctypes.c_ubyte
    lib.cpArbiterIsFirstContact.argtypes = [P]
    lib.cpArbiterCallWildcardBeginA.restype = ctypes.c_ubyte
    lib.cpArbiterCallWildcardBeginA.argtypes = [P, P]


class Callbacks:
    """The handlers of one space; counts[k] are the calls of each kind."""

    def __init__(self, lib, space):
        self.lib = lib
        self.counts = np.zeros(8, dtype=np.int64)
        self.impulse = [0.0, 0.0]
        c = self.counts

        def begin12(arb, sp, data):
            c[0] += 1
            return lib.cpArbiterCallWildcardBeginA(arb, sp)

        def pre12(arb, sp, data):
            c[1] += 1
            lib.cpArbiterSetFriction(arb, 0.5 * lib.cpArbiterGetFriction(arb))
            n = lib.cpArbiterGetNormal(arb)
            if n.y > 0.9:                    # contacts pushing straight up are dropped
                c[2] += 1
                return lib.cpArbiterIgnore(arb)
            return 1

        def begin23(arb, sp, data):
            c[3] += 1
            return 0 if c[3] % 3 == 0 else 1

        def post23(arb, sp, data):
            c[4] += 1
            j = lib.cpArbiterTotalImpulse(arb)
            self.impulse[0] += j.x
            self.impulse[1] += j.y

        def sep(arb, sp, data):
            c[5] += 1

        def wbegin(arb, sp, data):
            c[6] += 1
            return 1

        def wsep(arb, sp, data):
            c[7] += 1

        self.keep = [BEGIN(begin12), PRESOLVE(pre12), BEGIN(begin23), POSTSOLVE(post23), SEPARATE(sep),
                     BEGIN(wbegin), SEPARATE(wsep)]
        h = lib.cpSpaceAddCollisionHandler(space, 1, 2).contents
        h.beginFunc, h.preSolveFunc, h.separateFunc = self.keep[0], self.keep[1], self.keep[4]
        h = lib.cpSpaceAddCollisionHandler(space, 2, 3).contents
        h.beginFunc, h.postSolveFunc, h.separateFunc = self.keep[2], self.keep[3], self.keep[4]
        h = lib.cpSpaceAddWildcardHandler(space, 1).contents
        h.beginFunc, h.separateFunc = self.keep[5], self.keep[6]


def setup(lib, cfg, size):
    bind(lib)
    sc = Scene(lib, cfg, size)
    for i in range(sc.nshapes):
        lib.cpShapeSetCollisionType(lib.cpx_scene_shape(sc.h, i), 1 + i % 3)
    return sc, Callbacks(lib, sc.space)


CASES = [(1, 14, 300), (3, 600, 150), (6, 200, 200), (2, 800, 120)]
IDS = ["pyramid", "mixed", "joints", "circles"]


@pytest.mark.parametrize("cfg,size,steps", CASES, ids=IDS)
def test_oracle_bit_exact_with_handlers(ref_lib, oracle_lib, cfg, size, steps):
    r, rc = setup(ref_lib, cfg, size)
    o, oc = setup(oracle_lib, cfg, size)
    try:
        for s in range(steps):
            r.step(1 / 60)
            o.step(1 / 60)
            np.testing.assert_array_equal(oc.counts, rc.counts, err_msg="callback counts, step %d" % s)
            np.testing.assert_array_equal(o.bodies(), r.bodies(), err_msg="bodies, step %d" % s)
            np.testing.assert_array_equal(o.arbiters(), r.arbiters(), err_msg="arbiters, step %d" % s)
        assert oc.impulse == rc.impulse
        assert (rc.counts[[0, 1, 3, 4, 6]] > 0).all(), rc.counts
    finally:
        r.free()
        o.free()


@pytest.mark.gpu
@pytest.mark.parametrize("cfg,size,steps", CASES, ids=IDS)
def test_teacher_forced_with_handlers(gpu_lib, oracle_lib, cfg, size, steps):
    g, gc = setup(gpu_lib, cfg, size)
    o, oc = setup(oracle_lib, cfg, size)
    try:
        worst = 0.0
        for s in range(steps):
            if s > 0:
                force(g, o)
            g.step(1 / 60)
            o.step(1 / 60)
            check_gpu_error(gpu_lib)
            np.testing.assert_array_equal(gc.counts, oc.counts, err_msg="callback counts, step %d" % s)
            eb, ea, _ = compare_step(g, o, s)
            worst = max(worst, eb, ea)
        print("workload %d with handlers: calls %s; worst rel err %.3g" % (cfg, oc.counts.tolist(), worst))
        np.testing.assert_allclose(gc.impulse, oc.impulse, rtol=1e-9)
    finally:
        g.free()
        o.free()

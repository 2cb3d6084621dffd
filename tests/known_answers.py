"""Known-answer cases from the reference's own test suite, restated as
plain C-API calls so they run against any implementation of the API.

The reference ships them as Objective-C XCTest cases, which cannot be built
here; the inputs and expected values below are the ones those tests assert.
"""
import ctypes

import numpy as np

from chipmunk2d_gb300._lib import cpVect, cpTransform


def v(x, y):
    return cpVect(x, y)


def time_stepping(lib):
    """xcode/ObjectiveChipmunkTests/BodyTest.m:147-185 (testTimeSteping):
    gravity (0,-1), dt 1; a dynamic body accelerates before it moves, a
    kinematic body moves at its velocity, a static body stays put.
    Returns [(dyn_p, dyn_v, stat_p, stat_v, kin_p, kin_v)] after steps 1, 2."""
    space = lib.cpSpaceNew()
    lib.cpSpaceSetGravity(space, v(0, -1))
    dyn = lib.cpSpaceAddBody(space, lib.cpBodyNew(1.0, 1.0))
    stat = lib.cpSpaceAddBody(space, lib.cpBodyNewStatic())
    kin = lib.cpSpaceAddBody(space, lib.cpBodyNewKinematic())
    lib.cpBodySetVelocity(kin, v(1, 0))
    out = []
    for _ in range(2):
        lib.cpSpaceStep(space, 1.0)
        rec = []
        for b in (dyn, stat, kin):
            p = lib.cpBodyGetPosition(b)
            vel = lib.cpBodyGetVelocity(b)
            rec += [(p.x, p.y), (vel.x, vel.y)]
        out.append(tuple(rec))
    lib.cpSpaceFree(space)
    for b in (dyn, stat, kin):
        lib.cpBodyFree(b)
    return out


TIME_STEPPING_EXPECTED = [
    ((0.0, 0.0), (0.0, -1.0), (0.0, 0.0), (0.0, 0.0), (1.0, 0.0), (1.0, 0.0)),
    ((0.0, -1.0), (0.0, -2.0), (0.0, 0.0), (0.0, 0.0), (2.0, 0.0), (1.0, 0.0)),
]


def resting_ball(lib):
    """xcode/ObjectiveChipmunkTests/CallbacksTest.m:257-295
    (testPostStepRemoval) without its removal callback: a unit ball dropped
    from y=10 onto a static bar (-10,0)-(10,0) of radius 1 settles with its
    centre within 1.1*collisionSlop of y=2 after 100 steps of dt 0.01.
    Returns (final y, collisionSlop)."""
    space = lib.cpSpaceNew()
    lib.cpSpaceSetGravity(space, v(0, -100))
    bar = lib.cpSegmentShapeNew(lib.cpSpaceGetStaticBody(space), v(-10, 0), v(10, 0), 1.0)
    lib.cpSpaceAddShape(space, bar)
    ball = lib.cpBodyNew(1.0, lib.cpMomentForCircle(1.0, 0.0, 1.0, v(0, 0)))
    lib.cpSpaceAddBody(space, ball)
    lib.cpBodySetPosition(ball, v(0, 10))
    shape = lib.cpCircleShapeNew(ball, 1.0, v(0, 0))
    lib.cpSpaceAddShape(space, shape)
    for _ in range(100):
        lib.cpSpaceStep(space, 0.01)
    y = lib.cpBodyGetPosition(ball).y
    slop = lib.cpSpaceGetCollisionSlop(space)
    lib.cpSpaceFree(space)
    lib.cpShapeFree(shape)
    lib.cpShapeFree(bar)
    lib.cpBodyFree(ball)
    return y, slop


# xcode/ObjectiveChipmunkTests/ConvexTest.m:115-213 (testConvexHull):
# (input points, how many leading points to use, expected hull up to rotation)
HULL_CASES = [
    ([(0, 0), (1, 0)], 1, [(0, 0)]),
    ([(0, 0), (1, 0)], 2, [(0, 0), (1, 0)]),
    ([(0, 0), (1, 1), (1, 0)], 3, [(0, 0), (1, 0), (1, 1)]),
    ([(0, 0), (0, 1), (1, 1), (1, 0)], 4, [(0, 0), (1, 0), (1, 1), (0, 1)]),
    ([(0, 0), (1, 0), (0, 1), (1, 1)], 4, [(0, 0), (1, 0), (1, 1), (0, 1)]),
    ([(0.9, 0.5), (0.2, 0.3), (1.0, 0.0), (0.8, 0.6), (0.8, 0.4), (0.1, 0.4),
      (0.4, 0.1), (0.0, 0.0), (0.1, 0.9), (0.9, 0.6), (0.6, 0.2), (0.7, 0.3),
      (0.1, 0.3), (0.1, 0.5), (0.8, 0.3), (0.3, 0.8), (0.0, 1.0), (0.6, 0.7),
      (1.0, 1.0), (0.6, 0.8), (0.1, 0.7), (0.7, 0.9), (0.9, 0.2), (0.1, 0.1)],
     24, [(0, 0), (1, 0), (1, 1), (0, 1)]),
    ([(0, 0), (0, 1), (0, 2), (0, 3), (0, 4), (0, 5)], 6, [(0, 0), (0, 5)]),
    ([(0, 0), (1, 0), (2, 0), (3, 0), (4, 0), (5, 0)], 6, [(0, 0), (5, 0)]),
    ([(0, 0), (1, 1), (2, 2), (3, 3), (4, 4), (5, 5)], 6, [(0, 0), (5, 5)]),
    ([(0, 0)] * 5, 1, [(0, 0)]),
    ([(0, 0)] * 5, 3, [(0, 0)]),
    ([(0, 0)] * 5, 5, [(0, 0)]),
    ([(1.0, 0.0), (1.0, 0.5), (1.0, 1.0), (0.5, 1.0), (0.0, 1.0), (0.0, 0.5),
      (0.0, 0.0), (0.5, 0.0)], 8, [(0, 0), (1, 0), (1, 1), (0, 1)]),
    ([(0, 0), (0, 1), (1, 1), (1, 0), (0, 0), (0, 1), (1, 1), (1, 0)], 8,
     [(0, 0), (1, 0), (1, 1), (0, 1)]),
    ([(0, 0), (0, 0), (0, 1), (0, 1), (1, 1), (1, 1), (1, 0), (1, 0)], 8,
     [(0, 0), (1, 0), (1, 1), (0, 1)]),
]


def convex_hull(lib, pts):
    n = len(pts)
    arr = (cpVect * n)(*[cpVect(x, y) for x, y in pts])
    res = (cpVect * n)()
    first = ctypes.c_int(-1)
    k = lib.cpConvexHull(n, ctypes.cast(arr, ctypes.c_void_p), ctypes.cast(res, ctypes.c_void_p),
                         ctypes.byref(first), 0.0)
    return [(res[i].x, res[i].y) for i in range(k)], first.value


def check_hull_case(lib, pts, count, expected):
    """Assertions of ConvexTest.m:47-103 (AssertHull): for every rotation of
    the input, the hull has the expected vertices in the expected cyclic
    order, starts at input[first], has non-negative area, and is a fixed
    point of the hull routine."""
    pts = pts[:count]
    for rot in range(count):
        rotated = [pts[(i + rot) % count] for i in range(count)]
        hull, first = convex_hull(lib, rotated)
        assert len(hull) == len(expected)
        assert hull[0] == tuple(map(float, rotated[first]))
        exp = [tuple(map(float, e)) for e in expected]
        k = exp.index(hull[0])
        assert hull == [exp[(k + i) % len(exp)] for i in range(len(exp))]
        if len(hull) >= 3:
            arr = (cpVect * len(hull))(*[cpVect(x, y) for x, y in hull])
            assert lib.cpAreaForPoly(len(hull), ctypes.cast(arr, ctypes.c_void_p), 0.0) >= 0.0
        again, _ = convex_hull(lib, hull)
        assert again == hull


def random_hull_fixed_point(lib, n, seed):
    """ConvexTest.m:105-113 (AssertRandomHull): the hull of random points is
    a fixed point of the hull routine and has positive area."""
    rng = np.random.default_rng(seed)
    pts = [tuple(p) for p in rng.random((n, 2))]
    hull, _ = convex_hull(lib, pts)
    again, _ = convex_hull(lib, hull)
    assert again == hull
    arr = (cpVect * len(hull))(*[cpVect(x, y) for x, y in hull])
    assert lib.cpAreaForPoly(len(hull), ctypes.cast(arr, ctypes.c_void_p), 0.0) > 0.0
    return hull


IDENTITY = cpTransform(1.0, 0.0, 0.0, 1.0, 0.0, 0.0)

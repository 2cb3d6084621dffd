"""Features the GPU step does not run are refused, not run elsewhere: the
step reports CP_GPU_ERR_UNSUPPORTED through cpGpuGetLastError and leaves
the space unstepped (no CPU fallback).  The checks happen on the host
before any device work, so these run without a GPU."""
import ctypes
import os

import pytest

from chipmunk2d_gb300 import cpVect
from chipmunk2d_gb300._lib import LIB_PATH, bind

CP_GPU_ERR_UNSUPPORTED = 3

P, D = ctypes.c_void_p, ctypes.c_double
VELOCITY_FUNC = ctypes.CFUNCTYPE(None, P, cpVect, D, D)
PRESOLVE_FUNC = ctypes.CFUNCTYPE(None, P, P)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB_PATH):
        from chipmunk2d_gb300.build import build
        build()
    lib = bind(LIB_PATH, gpu=True)
    lib.cpSpaceSetSleepTimeThreshold.argtypes = [P, D]
    lib.cpBodySetVelocityUpdateFunc.argtypes = [P, VELOCITY_FUNC]
    lib.cpConstraintSetPreSolveFunc.argtypes = [P, PRESOLVE_FUNC]
    return lib


def one_body_space(lib):
    sp = lib.cpSpaceNew()
    lib.cpSpaceSetGravity(sp, cpVect(0, -100))
    b = lib.cpSpaceAddBody(sp, lib.cpBodyNew(1.0, 1.0))
    return sp, b


def refused(lib, sp, b):
    lib.cpGpuGetLastError()                          # clear
    p0 = lib.cpBodyGetPosition(b)
    lib.cpSpaceStep(sp, 1 / 60)
    err = lib.cpGpuGetLastError()
    p1 = lib.cpBodyGetPosition(b)
    return err, (p0.x, p0.y) == (p1.x, p1.y)


def test_sleeping_in_the_coloured_mode_is_refused(lib):
    """Sleeping runs in the exact-order mode, whose arbiter list order the
    sleeping edits follow."""
    sp, b = one_body_space(lib)
    lib.cpGpuSetSolverMode(sp, 1)
    lib.cpSpaceSetSleepTimeThreshold(sp, 0.5)
    err, unmoved = refused(lib, sp, b)
    assert err == CP_GPU_ERR_UNSUPPORTED and unmoved
    lib.cpSpaceFree(sp); lib.cpBodyFree(b)


def test_custom_velocity_functions_in_the_coloured_mode_are_refused(lib):
    """Velocity functions run on the host between the exact-order mode's
    device parts; the coloured mode refuses them."""
    sp, b = one_body_space(lib)
    lib.cpGpuSetSolverMode(sp, 1)
    cb = VELOCITY_FUNC(lambda body, g, damping, dt: None)
    lib.cpBodySetVelocityUpdateFunc(b, cb)
    err, unmoved = refused(lib, sp, b)
    assert err == CP_GPU_ERR_UNSUPPORTED and unmoved
    lib.cpSpaceFree(sp); lib.cpBodyFree(b)


POSITION_FUNC = ctypes.CFUNCTYPE(None, P, D)


def test_custom_position_functions_in_the_coloured_mode_are_refused(lib):
    lib.cpBodySetPositionUpdateFunc.argtypes = [P, POSITION_FUNC]
    sp, b = one_body_space(lib)
    lib.cpGpuSetSolverMode(sp, 1)
    cb = POSITION_FUNC(lambda body, dt: None)
    lib.cpBodySetPositionUpdateFunc(b, cb)
    err, unmoved = refused(lib, sp, b)
    assert err == CP_GPU_ERR_UNSUPPORTED and unmoved
    lib.cpSpaceFree(sp); lib.cpBodyFree(b)


def test_constraint_callbacks_in_the_coloured_mode_are_refused(lib):
    """The joints' pre/post-solve callbacks run on the host between the
    exact-order mode's device parts; the coloured mode refuses them."""
    sp, b = one_body_space(lib)
    lib.cpGpuSetSolverMode(sp, 1)
    c = lib.cpSpaceAddConstraint(sp, lib.cpPivotJointNew(lib.cpSpaceGetStaticBody(sp), b, cpVect(0, 0)))
    cb = PRESOLVE_FUNC(lambda con, space: None)
    lib.cpConstraintSetPreSolveFunc(c, cb)
    err, unmoved = refused(lib, sp, b)
    assert err == CP_GPU_ERR_UNSUPPORTED and unmoved
    lib.cpSpaceFree(sp); lib.cpConstraintFree(c); lib.cpBodyFree(b)


SPRING_FORCE = ctypes.CFUNCTYPE(D, P, D)


def test_custom_spring_force_is_refused(lib):
    """A damped spring with its own force function (host code) is refused;
    the default force runs on the GPU."""
    lib.cpDampedSpringNew.restype = P
    lib.cpDampedSpringNew.argtypes = [P, P, cpVect, cpVect, D, D, D]
    lib.cpDampedSpringSetSpringForceFunc.argtypes = [P, SPRING_FORCE]
    sp, b = one_body_space(lib)
    c = lib.cpSpaceAddConstraint(sp, lib.cpDampedSpringNew(lib.cpSpaceGetStaticBody(sp), b, cpVect(0, 0), cpVect(0, 0), 5.0, 10.0, 1.0))
    cb = SPRING_FORCE(lambda spring, dist: 0.0)
    lib.cpDampedSpringSetSpringForceFunc(c, cb)
    err, unmoved = refused(lib, sp, b)
    assert err == CP_GPU_ERR_UNSUPPORTED and unmoved
    lib.cpSpaceFree(sp); lib.cpConstraintFree(c); lib.cpBodyFree(b)


def test_handlers_and_the_hash_in_the_coloured_mode_are_refused(lib):
    """Collision handlers and the spatial hash follow the exact order's
    arbiter list and pair order; the coloured mode refuses both."""
    lib.cpSpaceAddCollisionHandler.restype = P
    lib.cpSpaceAddCollisionHandler.argtypes = [P, ctypes.c_size_t, ctypes.c_size_t]
    lib.cpSpaceUseSpatialHash.argtypes = [P, D, ctypes.c_int]
    for setup in (lambda sp: lib.cpSpaceAddCollisionHandler(sp, 1, 2), lambda sp: lib.cpSpaceUseSpatialHash(sp, 10.0, 100)):
        sp, b = one_body_space(lib)
        lib.cpGpuSetSolverMode(sp, 1)
        setup(sp)
        err, unmoved = refused(lib, sp, b)
        assert err == CP_GPU_ERR_UNSUPPORTED and unmoved
        lib.cpSpaceFree(sp); lib.cpBodyFree(b)


def test_sleeping_and_handlers_in_a_batch_are_refused(lib):
    """A batch steps its spaces without the host's parts of the step."""
    lib.cpGpuBatchNew.restype = P
    lib.cpGpuBatchAddSpace.argtypes = [P, P]
    lib.cpGpuBatchStep.argtypes = [P, D, ctypes.c_int, ctypes.c_int]
    lib.cpGpuBatchFree.argtypes = [P]
    lib.cpSpaceAddCollisionHandler.restype = P
    lib.cpSpaceAddCollisionHandler.argtypes = [P, ctypes.c_size_t, ctypes.c_size_t]
    for setup in (lambda sp: lib.cpSpaceSetSleepTimeThreshold(sp, 0.5), lambda sp: lib.cpSpaceAddCollisionHandler(sp, 1, 2)):
        sp, b = one_body_space(lib)
        setup(sp)
        batch = lib.cpGpuBatchNew()
        lib.cpGpuBatchAddSpace(batch, sp)
        lib.cpGpuGetLastError()
        assert lib.cpGpuBatchStep(batch, 1 / 60, 1, 0) == -1
        assert lib.cpGpuGetLastError() == CP_GPU_ERR_UNSUPPORTED
        lib.cpGpuBatchFree(batch)
        lib.cpSpaceFree(sp); lib.cpBodyFree(b)

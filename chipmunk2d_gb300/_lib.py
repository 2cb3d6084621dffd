"""ctypes binding of the Chipmunk2D C ABI.

``bind(path)`` loads any shared library that implements the Chipmunk2D
public API declared in ``include/chipmunk_gb300.h`` (the GPU drop-in built
from ``chipmunk2d_gb300/csrc``, or another implementation of the same API)
and attaches argument/return types to every entry point.  The library is
the product; this module is only the Python plumbing the tests and the
benchmark use to call it.
"""
import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_DIR = os.path.dirname(PKG_DIR)
LIB_PATH = os.path.join(PKG_DIR, "_build", "libchipmunk_gb300.so")
# the seeded workloads (csrc/scenes.c), linked against the product library
SCENES_PATH = os.path.join(PKG_DIR, "_build", "libcpx_scenes.so")
HEADER = os.path.join(REPO_DIR, "include", "chipmunk_gb300.h")


class cpVect(ctypes.Structure):
    _fields_ = [("x", ctypes.c_double), ("y", ctypes.c_double)]


class cpBB(ctypes.Structure):
    _fields_ = [("l", ctypes.c_double), ("b", ctypes.c_double),
                ("r", ctypes.c_double), ("t", ctypes.c_double)]


class cpTransform(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("a", "b", "c", "d", "tx", "ty")]


class cpShapeFilter(ctypes.Structure):
    _fields_ = [("group", ctypes.c_size_t), ("categories", ctypes.c_uint),
                ("mask", ctypes.c_uint)]


class _ContactPoint(ctypes.Structure):
    _fields_ = [("pointA", cpVect), ("pointB", cpVect), ("distance", ctypes.c_double)]


class cpContactPointSet(ctypes.Structure):
    _fields_ = [("count", ctypes.c_int), ("normal", cpVect),
                ("points", _ContactPoint * 2)]


P = ctypes.c_void_p
D = ctypes.c_double
I = ctypes.c_int
V = cpVect
ARBITER_ITER = ctypes.CFUNCTYPE(None, P, P, P)

# name: (restype, argtypes)
_API = {
    # misc (chipmunk.h)
    "cpMomentForCircle": (D, [D, D, D, V]),
    "cpAreaForCircle": (D, [D, D]),
    "cpMomentForSegment": (D, [D, V, V, D]),
    "cpAreaForSegment": (D, [V, V, D]),
    "cpMomentForPoly": (D, [D, I, P, V, D]),
    "cpAreaForPoly": (D, [I, P, D]),
    "cpCentroidForPoly": (V, [I, P]),
    "cpMomentForBox": (D, [D, D, D]),
    "cpMomentForBox2": (D, [D, cpBB]),
    "cpConvexHull": (I, [I, P, P, ctypes.POINTER(I), D]),
    # space
    "cpSpaceNew": (P, []),
    "cpSpaceFree": (None, [P]),
    "cpSpaceGetIterations": (I, [P]),
    "cpSpaceSetIterations": (None, [P, I]),
    "cpSpaceGetGravity": (V, [P]),
    "cpSpaceSetGravity": (None, [P, V]),
    "cpSpaceGetDamping": (D, [P]),
    "cpSpaceSetDamping": (None, [P, D]),
    "cpSpaceGetCollisionSlop": (D, [P]),
    "cpSpaceSetCollisionSlop": (None, [P, D]),
    "cpSpaceGetCollisionBias": (D, [P]),
    "cpSpaceSetCollisionBias": (None, [P, D]),
    "cpSpaceGetCollisionPersistence": (ctypes.c_uint, [P]),
    "cpSpaceSetCollisionPersistence": (None, [P, ctypes.c_uint]),
    "cpSpaceGetStaticBody": (P, [P]),
    "cpSpaceGetCurrentTimeStep": (D, [P]),
    "cpSpaceAddShape": (P, [P, P]),
    "cpSpaceAddBody": (P, [P, P]),
    "cpSpaceAddConstraint": (P, [P, P]),
    "cpSpaceStep": (None, [P, D]),
    # body
    "cpBodyNew": (P, [D, D]),
    "cpBodyNewStatic": (P, []),
    "cpBodyNewKinematic": (P, []),
    "cpBodyFree": (None, [P]),
    "cpBodyGetType": (I, [P]),
    "cpBodyGetMass": (D, [P]),
    "cpBodySetMass": (None, [P, D]),
    "cpBodyGetMoment": (D, [P]),
    "cpBodyGetPosition": (V, [P]),
    "cpBodySetPosition": (None, [P, V]),
    "cpBodyGetVelocity": (V, [P]),
    "cpBodySetVelocity": (None, [P, V]),
    "cpBodyGetAngle": (D, [P]),
    "cpBodySetAngle": (None, [P, D]),
    "cpBodyGetAngularVelocity": (D, [P]),
    "cpBodySetAngularVelocity": (None, [P, D]),
    "cpBodyGetRotation": (V, [P]),
    "cpBodyGetForce": (V, [P]),
    "cpBodySetForce": (None, [P, V]),
    "cpBodyLocalToWorld": (V, [P, V]),
    "cpBodyWorldToLocal": (V, [P, V]),
    "cpBodyEachArbiter": (None, [P, ARBITER_ITER, P]),
    # shapes
    "cpShapeFree": (None, [P]),
    "cpShapeGetBB": (cpBB, [P]),
    "cpShapeSetFriction": (None, [P, D]),
    "cpShapeGetFriction": (D, [P]),
    "cpShapeGetBody": (P, [P]),
    "cpShapeSetElasticity": (None, [P, D]),
    "cpShapeGetElasticity": (D, [P]),
    "cpCircleShapeNew": (P, [P, D, V]),
    "cpSegmentShapeNew": (P, [P, V, V, D]),
    "cpPolyShapeNew": (P, [P, I, P, cpTransform, D]),
    "cpPolyShapeNewRaw": (P, [P, I, P, D]),
    "cpBoxShapeNew": (P, [P, D, D, D]),
    "cpPolyShapeGetCount": (I, [P]),
    "cpPolyShapeGetVert": (V, [P, I]),
    # sleeping
    "cpSpaceSetSleepTimeThreshold": (None, [P, D]),
    "cpSpaceGetSleepTimeThreshold": (D, [P]),
    "cpSpaceSetIdleSpeedThreshold": (None, [P, D]),
    "cpBodyIsSleeping": (ctypes.c_ubyte, [P]),
    "cpBodyActivate": (None, [P]),
    "cpBodySleep": (None, [P]),
    # constraints
    "cpConstraintFree": (None, [P]),
    "cpConstraintGetImpulse": (D, [P]),
    "cpConstraintSetCollideBodies": (None, [P, ctypes.c_ubyte]),
    "cpPivotJointNew": (P, [P, P, V]),
    "cpPinJointNew": (P, [P, P, V, V]),
    "cpSlideJointNew": (P, [P, P, V, V, D, D]),
    # arbiters
    "cpArbiterTotalImpulse": (V, [P]),
    "cpArbiterGetCount": (I, [P]),
    "cpArbiterGetContactPointSet": (cpContactPointSet, [P]),
    # seeded workloads (scenes.c)
    "cpx_scene_build": (P, [I, I, ctypes.c_ulonglong]),
    "cpx_scene_space": (P, [P]),
    "cpx_scene_body_count": (I, [P]),
    "cpx_scene_shape_count": (I, [P]),
    "cpx_scene_constraint_count": (I, [P]),
    "cpx_scene_body": (P, [P, I]),
    "cpx_scene_shape": (P, [P, I]),
    "cpx_scene_constraint": (P, [P, I]),
    "cpx_scene_dump_public": (I, [P, P]),
    "cpx_scene_dump_impulses": (I, [P, P]),
    "cpx_scene_step": (None, [P, D, I]),
    "cpx_space_set_hasty": (I, [P, I]),
    "cpx_scene_free": (None, [P]),
    "cpx_scene_edit": (I, [P, I, ctypes.c_ulonglong]),
    "cpx_scene_queries": (I, [P, I, I, P, I]),
    "cpx_batch_sizes": (None, [I, ctypes.c_ulonglong, P]),
    # state export (shared record layouts)
    "cpx_dump_bodies": (I, [P, P, I]),
    "cpx_dump_arbiters": (I, [P, P, I]),
    "cpx_dump_constraints": (I, [P, P, I]),
    "cpx_set_bodies": (I, [P, P, I]),
    "cpx_dump_candidates": (I, [P, P, I]),
}

# GPU-only entry points (libchipmunk_gb300.so)
_GPU_API = {
    "cpGpuSetSolverMode": (None, [P, I]),
    "cpGpuGetSolverMode": (I, [P]),
    "cpGpuGetLastError": (I, []),
    "cpGpuGetLastErrorString": (ctypes.c_char_p, []),
    "cpGpuSetStream": (None, [P]),
    "cpGpuSpaceSync": (None, [P]),
    "cpGpuBatchNew": (P, []),
    "cpGpuBatchFree": (None, [P]),
    "cpGpuBatchAddSpace": (I, [P, P]),
    "cpGpuBatchStep": (I, [P, D, I, I]),
    "cpGpuBatchGetTuning": (I, [P, P]),
    "cpGpuSetAutotune": (None, [I]),
    "cpGpuRolloutForward": (I, [P, D, I, I]),
    "cpGpuRolloutBackward": (I, [P, P, P, P, P, P, P]),
    "cpGpuRolloutBackwardFull": (I, [P] * 12),
    "cpGpuDebugRolloutTimes": (I, [P, P]),
    "cpGpuDebugSetRolloutRecording": (None, [I]),
    "cpGpuDebugBodies": (I, [P, P, I]),
    "cpGpuDebugArbiters": (I, [P, P, I]),
    "cpGpuDebugConstraints": (I, [P, P, I]),
    "cpGpuDebugSetBodies": (I, [P, P, I]),
    "cpGpuDebugSetImpulses": (I, [P, P, I, P, I]),
    "cpGpuDebugCandidates": (I, [P, P, I]),
    "cpGpuSetTiming": (None, [I]),
    "cpGpuDebugSetWholeGridSolve": (None, [I]),
    "cpGpuDebugSetTreeStaging": (None, [I]),
    "cpGpuDebugSetSolveShape": (None, [I, I]),
    "cpGpuDebugSetSolveLayout": (None, [I]),
    "cpGpuDebugSetFlowSolve": (None, [I]),
    "cpGpuDebugSetFlowWaitLimit": (None, [I, I]),
    "cpGpuDebugSetCapacities": (None, [I, I, I, I]),
    "cpGpuDebugSetWarmStartGather": (None, [I]),
    "cpGpuDebugSetParallelMarking": (None, [I]),
    "cpGpuDebugSetCoopBlocks": (None, [I]),
    "cpGpuGetPhaseTimes": (I, [P, P, I]),
    "cpGpuSolverQuality": (I, [P, I, D, I, P]),
    "cpGpuSpaceGetBodyStates": (I, [P, P, I]),
    "cpGpuGetStepStats": (I, [P, P, I]),
    "cpGpuGetLaunchCount": (ctypes.c_longlong, [I]),
    "cpGpuSolveSchedule": (I, [P, P, I, I, P, P, P, P]),
    "cpGpuSolveScheduleNoAlloc": (I, [P, P, I, I, P, P, P, P]),
}

BODY_REC, ARB_REC, CONS_REC = 18, 34, 8


def bind(path, gpu=False):
    """Load the shared library at ``path`` and attach ctypes signatures."""
    lib = ctypes.CDLL(path)
    table = dict(_API)
    if gpu:
        table.update(_GPU_API)
    for name, (res, args) in table.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue
        fn.restype = res
        fn.argtypes = args
    return lib


def load_gpu_library():
    """Load the in-tree GPU drop-in together with the seeded workloads.

    The workloads live in libcpx_scenes.so, which links against
    libchipmunk_gb300.so; symbol lookup through its handle also searches the
    product library it depends on, so one handle serves both.  Raises if
    they have not been built."""
    for path in (LIB_PATH, SCENES_PATH):
        if not os.path.exists(path):
            raise RuntimeError(
                "%s is not built; run "
                "`python -c 'import __graft_entry__ as g; g.build()'`" % os.path.basename(path))
    # RTLD_LOCAL (ctypes' default): with the product in the global scope,
    # another implementation of the API loaded later (the oracle) would
    # bind its own calls to the product's symbols
    return bind(SCENES_PATH, gpu=True)


def load_product_library():
    """The product library alone (libchipmunk_gb300.so), for checks of what
    it exports."""
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libchipmunk_gb300.so is not built")
    return bind(LIB_PATH, gpu=True)


class Scene:
    """A seeded workload built through the C API of a given library."""

    def __init__(self, lib, config, size=0, seed=None):
        self.lib = lib
        self.h = lib.cpx_scene_build(config, size, config if seed is None else seed)
        if not self.h:
            raise ValueError("unknown workload %d" % config)
        self.space = lib.cpx_scene_space(self.h)
        self.nbodies = lib.cpx_scene_body_count(self.h)
        self.nshapes = lib.cpx_scene_shape_count(self.h)
        self.nconstraints = lib.cpx_scene_constraint_count(self.h)

    def step(self, dt, steps=1):
        self.lib.cpx_scene_step(self.h, dt, steps)

    def bodies(self):
        # the space's dynamic bodies now (objects may have been added or removed)
        cap = self.lib.cpx_dump_bodies(self.space, None, 0)
        out = np.zeros(BODY_REC * max(cap, 1))
        n = self.lib.cpx_dump_bodies(self.space, out.ctypes.data, cap)
        return out[:BODY_REC * n].reshape(n, BODY_REC)

    def edit(self, round_, seed):
        """One round of deterministic edits between steps (cpx_scene_edit):
        removals, additions, constraint churn and body-type changes."""
        n = self.lib.cpx_scene_edit(self.h, round_, seed)
        self.nbodies = self.lib.cpx_scene_body_count(self.h)
        self.nshapes = self.lib.cpx_scene_shape_count(self.h)
        self.nconstraints = self.lib.cpx_scene_constraint_count(self.h)
        return n

    def set_bodies(self, arr):
        arr = np.ascontiguousarray(arr, dtype=np.float64)
        return self.lib.cpx_set_bodies(self.space, arr.ctypes.data, arr.shape[0])

    def set_impulses(self, arbs, cons):
        """Warm-start state (GPU library only): accumulated impulses of the
        last solve list's arbiters and of the constraints, from another
        implementation's dumps.  Returns the count of skipped records."""
        arbs = np.ascontiguousarray(arbs, dtype=np.float64)
        cons = np.ascontiguousarray(cons, dtype=np.float64)
        return self.lib.cpGpuDebugSetImpulses(self.space, arbs.ctypes.data, arbs.shape[0],
                                              cons.ctypes.data, cons.shape[0])

    def arbiters(self, cap=None):
        cap = cap or max(4 * self.nshapes + 16, 64)
        while True:
            out = np.zeros(ARB_REC * cap)
            n = self.lib.cpx_dump_arbiters(self.space, out.ctypes.data, cap)
            if n <= cap:
                return out[:ARB_REC * n].reshape(n, ARB_REC)
            cap = n

    def constraints(self):
        cap = self.lib.cpx_dump_constraints(self.space, None, 0)
        out = np.zeros(CONS_REC * max(cap, 1))
        n = self.lib.cpx_dump_constraints(self.space, out.ctypes.data, cap)
        return out[:CONS_REC * n].reshape(n, CONS_REC)

    def candidates(self, cap=None):
        cap = cap or max(16 * self.nshapes + 64, 64)
        out = np.zeros(2 * cap, dtype=np.int32)
        n = self.lib.cpx_dump_candidates(self.space, out.ctypes.data, cap)
        pairs = out[:2 * min(n, cap)].reshape(-1, 2)
        return set(map(tuple, pairs.tolist()))

    def queries(self, seed, nq):
        """nq seeded spatial queries through the public API (scenes.c,
        cpx_scene_queries): one row of 8 per callback or result."""
        cap = 64 * nq + 64
        while True:
            out = np.zeros(8 * cap)
            n = self.lib.cpx_scene_queries(self.h, seed, nq, out.ctypes.data, cap)
            if n <= cap:
                return out[:8 * n].reshape(n, 8)
            cap = n

    def public(self):
        out = np.zeros(8 * max(self.nbodies, 1))
        self.lib.cpx_scene_dump_public(self.h, out.ctypes.data)
        return out[:8 * self.nbodies].reshape(self.nbodies, 8)

    def impulses(self):
        out = np.zeros(2 * max(self.nbodies, 1))
        self.lib.cpx_scene_dump_impulses(self.h, out.ctypes.data)
        return out[:2 * self.nbodies].reshape(self.nbodies, 2)

    def free(self):
        if self.h:
            self.lib.cpx_scene_free(self.h)
            self.h = None

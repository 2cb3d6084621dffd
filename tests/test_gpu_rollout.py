"""Differentiable rollout (cpGpuRolloutForward / cpGpuRolloutBackward).

The reverse pass's gradients of L = sum |p_final - target|^2 are compared
with central finite differences of the forward: of the GPU forward (the
same batch stepped by cpGpuBatchStep with one parameter moved by +-h) and
of the CPU oracle.  The scene is the rollout workload (circles and boxes
dropped onto a ground segment, 10 iterations, dt = 1/120), with fewer
worlds and bodies than the benchmark so that the finite differences, two
full rollouts per parameter, stay cheap.
"""
import ctypes

import numpy as np
import pytest

from chipmunk2d_gb300 import Scene, cpVect

pytestmark = pytest.mark.gpu

DT = 1 / 120
WORLDS, SIZE = 6, 16


def make(lib, seeds):
    return [Scene(lib, 5, SIZE, seed=s) for s in seeds]


def positions(scenes):
    return np.concatenate([sc.bodies()[:, 0:2] for sc in scenes])


def targets(n):
    return np.random.default_rng(4).normal(0.0, 10.0, size=(n, 2))


def loss(p, t):
    return float(np.sum((p - t) ** 2))


class Param:
    """One differentiable parameter of the batch: kind, world, index, component."""

    def __init__(self, kind, world, index, comp=0):
        self.kind, self.world, self.index, self.comp = kind, world, index, comp

    def apply(self, lib, scenes, h):
        sc = scenes[self.world]
        if self.kind in ("v", "w", "m"):
            body = lib.cpx_scene_body(sc.h, self.index)
            if self.kind == "v":
                v = lib.cpBodyGetVelocity(body)
                lib.cpBodySetVelocity(body, cpVect(v.x + (h if self.comp == 0 else 0.0), v.y + (h if self.comp == 1 else 0.0)))
            elif self.kind == "w":
                lib.cpBodySetAngularVelocity(body, lib.cpBodyGetAngularVelocity(body) + h)
            else:
                lib.cpBodySetMass(body, lib.cpBodyGetMass(body) + h)
        else:
            shape = lib.cpx_scene_shape(sc.h, self.index)
            if self.kind == "e":
                lib.cpShapeSetElasticity(shape, lib.cpShapeGetElasticity(shape) + h)
            else:
                lib.cpShapeSetFriction(shape, lib.cpShapeGetFriction(shape) + h)

    def grad(self, g):
        b = self.world * SIZE + self.index
        s = self.world * (SIZE + 1) + self.index
        return {"v": g["v0"][2 * b + self.comp], "w": g["w0"][b], "m": g["m"][b],
                "e": g["e"][s], "u": g["u"][s]}[self.kind]


def gpu_loss(lib, seeds, steps, t, param=None, h=0.0):
    scenes = make(lib, seeds)
    if param is not None:
        param.apply(lib, scenes, h)
    batch = lib.cpGpuBatchNew()
    for sc in scenes:
        lib.cpGpuBatchAddSpace(batch, sc.space)
    assert lib.cpGpuBatchStep(batch, DT, steps, 0) == 0
    L = loss(positions(scenes), t)
    lib.cpGpuBatchFree(batch)
    for sc in scenes:
        sc.free()
    return L


def oracle_loss(lib, seeds, steps, t, param=None, h=0.0):
    scenes = make(lib, seeds)
    if param is not None:
        param.apply(lib, scenes, h)
    for sc in scenes:
        sc.step(DT, steps)
    L = loss(positions(scenes), t)
    for sc in scenes:
        sc.free()
    return L


def rollout_grads(lib, seeds, steps, K, t):
    scenes = make(lib, seeds)
    batch = lib.cpGpuBatchNew()
    for sc in scenes:
        lib.cpGpuBatchAddSpace(batch, sc.space)
    assert lib.cpGpuRolloutForward(batch, DT, steps, K) == 0, lib.cpGpuGetLastErrorString()
    p = positions(scenes)
    nd = len(p)
    ns = sum(sc.nshapes for sc in scenes)
    dLdp = np.ascontiguousarray(2.0 * (p - t)).ravel()
    g = {"v0": np.zeros(2 * nd), "w0": np.zeros(nd), "m": np.zeros(nd), "e": np.zeros(ns), "u": np.zeros(ns)}
    rc = lib.cpGpuRolloutBackward(batch, dLdp.ctypes.data, g["v0"].ctypes.data, g["w0"].ctypes.data,
                                  g["m"].ctypes.data, g["e"].ctypes.data, g["u"].ctypes.data)
    assert rc == 0, lib.cpGpuGetLastErrorString()
    # the batch is left in the forward's final state
    np.testing.assert_array_equal(positions(scenes), p)
    lib.cpGpuBatchFree(batch)
    for sc in scenes:
        sc.free()
    return g, loss(p, t)


def test_one_step_free_fall_gradient_is_exact(gpu_lib):
    """Before the first contact, p1 = p0 + v0*dt, so dL/dv0 = 2 (p1 - t) dt."""
    seeds = [4000 + i for i in range(WORLDS)]
    scenes = make(gpu_lib, seeds)
    p0 = positions(scenes)
    v0 = np.concatenate([sc.bodies()[:, 2:4] for sc in scenes])
    for sc in scenes:
        sc.free()
    t = targets(len(p0))
    g, _ = rollout_grads(gpu_lib, seeds, 1, 1, t)
    p1 = p0 + v0 * DT
    np.testing.assert_allclose(g["v0"].reshape(-1, 2), 2.0 * (p1 - t) * DT, rtol=1e-12, atol=1e-12)


def test_gradients_do_not_depend_on_the_checkpoint_interval(gpu_lib):
    seeds = [4000 + i for i in range(WORLDS)]
    t = targets(WORLDS * SIZE)
    a, La = rollout_grads(gpu_lib, seeds, 60, 60, t)
    b, Lb = rollout_grads(gpu_lib, seeds, 60, 16, t)
    assert La == Lb
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_recorded_and_replayed_segments_give_the_same_gradients(gpu_lib):
    """The reverse pass recomputes a segment's solver iterations from what
    the forward recorded, or replays the segment from its checkpoint when
    nothing was recorded; the gradients are bit-identical."""
    seeds = [4000 + i for i in range(WORLDS)]
    t = targets(WORLDS * SIZE)
    a, La = rollout_grads(gpu_lib, seeds, 60, 16, t)
    gpu_lib.cpGpuDebugSetRolloutRecording(0)
    try:
        b, Lb = rollout_grads(gpu_lib, seeds, 60, 16, t)
    finally:
        gpu_lib.cpGpuDebugSetRolloutRecording(1)
    assert La == Lb
    for k in a:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)


def test_gradients_are_deterministic_at_scale(gpu_lib):
    """Arbiters created between checkpoints can take other table slots in
    the replay than in the forward; the carried impulse adjoints follow
    them by key, so two runs give identical gradients."""
    global WORLDS, SIZE
    saved = WORLDS, SIZE
    WORLDS, SIZE = 256, 64
    try:
        seeds = [4000 + i for i in range(WORLDS)]
        t = targets(WORLDS * SIZE)
        a, La = rollout_grads(gpu_lib, seeds, 120, 16, t)
        b, Lb = rollout_grads(gpu_lib, seeds, 120, 16, t)
        assert La == Lb
        for k in a:
            np.testing.assert_array_equal(a[k], b[k], err_msg=k)
    finally:
        WORLDS, SIZE = saved


def sample_params():
    rng = np.random.default_rng(11)
    ps = []
    for _ in range(16):
        ps.append(Param("v", int(rng.integers(WORLDS)), int(rng.integers(SIZE)), int(rng.integers(2))))
    for _ in range(6):
        ps.append(Param("w", int(rng.integers(WORLDS)), int(rng.integers(SIZE))))
    for _ in range(6):
        ps.append(Param("m", int(rng.integers(WORLDS)), int(rng.integers(SIZE))))
    for _ in range(6):
        ps.append(Param("e", int(rng.integers(WORLDS)), int(rng.integers(SIZE + 1))))
    for _ in range(6):
        ps.append(Param("u", int(rng.integers(WORLDS)), int(rng.integers(SIZE + 1))))
    return ps


STEPS = 150


def test_gradients_match_gpu_finite_differences(gpu_lib):
    """Central differences at h = 1e-6 and 1e-7: their distance u bounds
    the differences' own error.  Where u > 1e-2 |fd| a contact event lies
    within the step and the loss is not smooth there (skipped).  Elsewhere
    the adjoint must agree within max(1e-6 |fd|, u), and where the
    differences are resolved to 1e-6 (u <= 1e-6 |fd|) to 1e-6 relative."""
    seeds = [4000 + i for i in range(WORLDS)]
    t = targets(WORLDS * SIZE)
    g, L0 = rollout_grads(gpu_lib, seeds, STEPS, 16, t)
    assert gpu_loss(gpu_lib, seeds, STEPS, t) == L0
    rows = []
    for p in sample_params():
        fd = []
        for h in (1e-6, 1e-7):
            fd.append((gpu_loss(gpu_lib, seeds, STEPS, t, p, h) - gpu_loss(gpu_lib, seeds, STEPS, t, p, -h)) / (2 * h))
        rows.append((p, p.grad(g), fd[0], fd[1]))
    smooth, resolved, bad = 0, 0, []
    for p, adj, f6, f7 in rows:
        u = abs(f6 - f7)
        kink = u > 1e-2 * abs(f6)
        err = abs(adj - f6) / max(abs(f6), 1e-300)
        print("%s w%d i%d c%d adjoint %+.10e fd %+.10e %+.10e rel %.2e%s" % (
            p.kind, p.world, p.index, p.comp, adj, f6, f7, err, "  (contact event)" if kink else ""))
        if kink:
            continue
        smooth += 1
        if abs(adj - f6) > max(1e-6 * abs(f6), u):
            bad.append((p.kind, p.world, p.index, p.comp, adj, f6, f7))
        if u <= 1e-6 * abs(f6) and f6 != 0.0:
            resolved += 1
            if err > 1e-6:
                bad.append(("resolved", p.kind, p.world, p.index, p.comp, adj, f6, f7))
    assert smooth >= 0.75 * len(rows), smooth
    assert resolved >= 5, resolved
    assert not bad, bad


def test_gradients_match_oracle_finite_differences(gpu_lib, oracle_lib):
    """The CPU reference's forward (the oracle) gives the same finite
    differences: the GPU forward agrees with it to ~1e-12 per step."""
    seeds = [4000 + i for i in range(2)]
    global WORLDS
    saved = WORLDS
    WORLDS = 2
    try:
        t = targets(WORLDS * SIZE)
        g, L0 = rollout_grads(gpu_lib, seeds, 40, 16, t)
        params = [Param("v", 0, 3, 0), Param("v", 1, 9, 1), Param("w", 0, 12), Param("m", 1, 2), Param("u", 0, 0), Param("e", 1, 5)]
        for p in params:
            h = 1e-5
            fd = (oracle_loss(oracle_lib, seeds, 40, t, p, h) - oracle_loss(oracle_lib, seeds, 40, t, p, -h)) / (2 * h)
            adj = p.grad(g)
            assert abs(adj - fd) <= 1e-4 * max(abs(fd), 1.0), (p.kind, adj, fd)
    finally:
        WORLDS = saved


CV, CA = 0.5, 100.0


def full_loss(scenes, t):
    b = np.concatenate([sc.bodies() for sc in scenes])
    p, v, a = b[:, 0:2], b[:, 2:4], b[:, 4]
    return float(np.sum((p - t) ** 2) + CV*np.sum(v ** 2) + CA*np.sum(a ** 2))


def apply_pose(lib, scenes, kind, world, index, comp, h):
    body = lib.cpx_scene_body(scenes[world].h, index)
    if kind == "p":
        q = lib.cpBodyGetPosition(body)
        lib.cpBodySetPosition(body, cpVect(q.x + (h if comp == 0 else 0.0), q.y + (h if comp == 1 else 0.0)))
    elif kind == "a":
        lib.cpBodySetAngle(body, lib.cpBodyGetAngle(body) + h)
    else:
        Param(kind, world, index, comp).apply(lib, scenes, h)


def gpu_full_loss(lib, seeds, steps, t, p=None, h=0.0):
    scenes = make(lib, seeds)
    if p is not None:
        apply_pose(lib, scenes, *p, h)
    batch = lib.cpGpuBatchNew()
    for sc in scenes:
        lib.cpGpuBatchAddSpace(batch, sc.space)
    assert lib.cpGpuBatchStep(batch, DT, steps, 0) == 0
    L = full_loss(scenes, t)
    lib.cpGpuBatchFree(batch)
    for sc in scenes:
        sc.free()
    return L


def test_full_gradients_match_gpu_finite_differences(gpu_lib):
    """cpGpuRolloutBackwardFull with seeds on the final positions, angles and
    velocities (L = sum |p - t|^2 + 0.5 |v|^2 + 100 a^2): the gradients with
    respect to the initial positions, angles, velocities and angular
    velocities agree with central differences of the GPU forward, with the
    same screening as the position-only test."""
    seeds = [4000 + i for i in range(WORLDS)]
    t = targets(WORLDS * SIZE)
    scenes = make(gpu_lib, seeds)
    batch = gpu_lib.cpGpuBatchNew()
    for sc in scenes:
        gpu_lib.cpGpuBatchAddSpace(batch, sc.space)
    assert gpu_lib.cpGpuRolloutForward(batch, DT, STEPS, 16) == 0, gpu_lib.cpGpuGetLastErrorString()
    L0 = full_loss(scenes, t)
    b = np.concatenate([sc.bodies() for sc in scenes])
    n = len(b)
    sp = np.ascontiguousarray(2.0 * (b[:, 0:2] - t)).ravel()
    sv = np.ascontiguousarray(2.0 * CV * b[:, 2:4]).ravel()
    sa = np.ascontiguousarray(2.0 * CA * b[:, 4])
    g = {k: np.zeros(s) for k, s in (("p", 2 * n), ("a", n), ("v", 2 * n), ("w", n))}
    rc = gpu_lib.cpGpuRolloutBackwardFull(batch, sp.ctypes.data, sa.ctypes.data, sv.ctypes.data, None,
                                          g["p"].ctypes.data, g["a"].ctypes.data, g["v"].ctypes.data, g["w"].ctypes.data,
                                          None, None, None)
    assert rc == 0, gpu_lib.cpGpuGetLastErrorString()
    gpu_lib.cpGpuBatchFree(batch)
    for sc in scenes:
        sc.free()
    assert gpu_full_loss(gpu_lib, seeds, STEPS, t) == L0
    rng = np.random.default_rng(23)
    params = [(k, int(rng.integers(WORLDS)), int(rng.integers(SIZE)), int(rng.integers(2)))
              for k in ["p"] * 10 + ["a"] * 8 + ["v"] * 6 + ["w"] * 6]
    smooth, resolved, bad = 0, 0, []
    for kind, w, i, c in params:
        fd = [(gpu_full_loss(gpu_lib, seeds, STEPS, t, (kind, w, i, c), h) -
               gpu_full_loss(gpu_lib, seeds, STEPS, t, (kind, w, i, c), -h)) / (2 * h) for h in (1e-6, 1e-7)]
        k = w * SIZE + i
        adj = g[kind][2 * k + c] if kind in ("p", "v") else g[kind][k]
        u = abs(fd[0] - fd[1])
        kink = u > 1e-2 * abs(fd[0])
        print("%s w%d i%d c%d adjoint %+.10e fd %+.10e %+.10e%s" % (kind, w, i, c, adj, fd[0], fd[1], "  (contact event)" if kink else ""))
        if kink:
            continue
        smooth += 1
        if abs(adj - fd[0]) > max(1e-6 * abs(fd[0]), u):
            bad.append((kind, w, i, c, adj, fd[0], fd[1]))
        if u <= 1e-6 * abs(fd[0]) and fd[0] != 0.0:
            resolved += 1
            if abs(adj - fd[0]) > 1e-6 * abs(fd[0]):
                bad.append(("resolved", kind, w, i, c, adj, fd[0], fd[1]))
    assert smooth >= 0.7 * len(params), smooth
    assert resolved >= 4, resolved
    assert not bad, bad

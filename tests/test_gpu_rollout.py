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


def gpu_final(lib, seeds, steps, param=None, h=0.0):
    """Final body records of the GPU forward with one parameter moved by h."""
    scenes = make(lib, seeds)
    if param is not None:
        param.apply(lib, scenes, h)
    batch = lib.cpGpuBatchNew()
    for sc in scenes:
        lib.cpGpuBatchAddSpace(batch, sc.space)
    assert lib.cpGpuBatchStep(batch, DT, steps, 0) == 0
    b = np.concatenate([sc.bodies() for sc in scenes])
    lib.cpGpuBatchFree(batch)
    for sc in scenes:
        sc.free()
    return b


def gpu_loss(lib, seeds, steps, t, param=None, h=0.0):
    return loss(gpu_final(lib, seeds, steps, param, h)[:, 0:2], t)


# Central differences of L = sum |p - t|^2 formed from the state itself:
# L(+h) - L(-h) = sum (p+ - p-) (p+ + p- - 2t), so the rounding of a loss of
# ~1e5 (one unit in the last place is ~3e-11, i.e. ~1e-5 absolute in a
# difference at h = 1e-6) does not enter.  Three step sizes bound the
# differences' own error by their spread u (two sizes can agree by chance).
FD_STEPS = (1e-5, 1e-6, 1e-7)


def central_difference(final_of, t, extra=None):
    """final_of(h) -> final records.  Returns the central differences at
    FD_STEPS of sum |p - t|^2, plus extra(plus, minus), the difference of
    any further loss terms."""
    out = []
    for h in FD_STEPS:
        bp, bm = final_of(h), final_of(-h)
        pp, pm = bp[:, 0:2], bm[:, 0:2]
        dl = float(np.sum((pp - pm) * (pp + pm - 2.0 * t)))
        if extra is not None:
            dl += extra(bp, bm)
        out.append(dl / (2 * h))
    return out


def fd_verdict(adj, fds):
    """(kink, resolved, ok, u): a contact event inside the step when the two
    smaller sizes disagree by more than 1e-2; otherwise the adjoint must lie
    within max(1e-6 |fd|, u) of the h = 1e-6 difference, u being the spread
    of the three; 'resolved' when u <= 1e-6 |fd|."""
    f5, f6, f7 = fds
    kink = abs(f6 - f7) > 1e-2 * abs(f6)
    u = max(abs(f5 - f6), abs(f6 - f7), abs(f5 - f7))
    resolved = (not kink) and f6 != 0.0 and u <= 1e-6 * abs(f6)
    ok = kink or abs(adj - f6) <= max(1e-6 * abs(f6), u)
    return kink, resolved, ok, u


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
    """Central differences at three step sizes (FD_STEPS, fd_verdict): where
    the two smaller ones disagree by more than 1e-2 a contact event lies
    within the step and the loss is not smooth there (skipped).  Elsewhere
    the adjoint must agree within max(1e-6 |fd|, u), u the differences'
    spread, and to 1e-6 relative where they are resolved to 1e-6."""
    seeds = [4000 + i for i in range(WORLDS)]
    t = targets(WORLDS * SIZE)
    g, L0 = rollout_grads(gpu_lib, seeds, STEPS, 16, t)
    assert gpu_loss(gpu_lib, seeds, STEPS, t) == L0
    smooth, resolved, bad = 0, 0, []
    params = sample_params()
    for p in params:
        adj = p.grad(g)
        fds = central_difference(lambda h: gpu_final(gpu_lib, seeds, STEPS, p, h), t)
        kink, res, ok, u = fd_verdict(adj, fds)
        err = abs(adj - fds[1]) / max(abs(fds[1]), 1e-300)
        print("%s w%d i%d c%d adjoint %+.10e fd %+.10e %+.10e %+.10e rel %.2e u %.1e%s" % (
            p.kind, p.world, p.index, p.comp, adj, *fds, err, u / max(abs(fds[1]), 1e-300), "  (contact event)" if kink else ""))
        smooth += not kink
        resolved += res
        if not ok:
            bad.append((p.kind, p.world, p.index, p.comp, adj, fds))
    assert smooth >= 0.75 * len(params), smooth
    assert resolved >= 5, resolved
    assert not bad, bad


def test_gradients_match_oracle_finite_differences(gpu_lib, oracle_lib):
    """The CPU reference's forward (the oracle) gives the same finite
    differences as the GPU's: the GPU adjoint agrees with central
    differences of the oracle under the same rule (fd_verdict: 1e-6
    relative where the differences are resolved to 1e-6), on 18 parameters
    of 3 worlds over 60 steps."""
    global WORLDS
    saved = WORLDS
    WORLDS = 3
    steps = 60
    try:
        seeds = [4000 + i for i in range(WORLDS)]
        t = targets(WORLDS * SIZE)
        g, L0 = rollout_grads(gpu_lib, seeds, steps, 16, t)
        rng = np.random.default_rng(29)
        params = [Param(k, int(rng.integers(WORLDS)), int(rng.integers(SIZE + (k in "eu"))), int(rng.integers(2)))
                  for k in ["v"] * 6 + ["w"] * 3 + ["m"] * 3 + ["u"] * 3 + ["e"] * 3]

        def final_of(p):
            def run(h):
                scenes = make(oracle_lib, seeds)
                p.apply(oracle_lib, scenes, h)
                for sc in scenes:
                    sc.step(DT, steps)
                b = np.concatenate([sc.bodies() for sc in scenes])
                for sc in scenes:
                    sc.free()
                return b
            return run

        smooth, resolved, bad = 0, 0, []
        for p in params:
            adj = p.grad(g)
            fds = central_difference(final_of(p), t)
            kink, res, ok, u = fd_verdict(adj, fds)
            print("%s w%d i%d c%d adjoint %+.10e oracle fd %+.10e %+.10e %+.10e u %.1e%s" % (
                p.kind, p.world, p.index, p.comp, adj, *fds, u / max(abs(fds[1]), 1e-300), "  (contact event)" if kink else ""))
            smooth += not kink
            resolved += res
            if not ok:
                bad.append((p.kind, p.world, p.index, p.comp, adj, fds))
        assert smooth >= 0.7 * len(params), smooth
        assert resolved >= 4, resolved
        assert not bad, bad
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

    def extra(bp, bm):
        # the velocity and angle terms of L, in the same difference form
        vp, vm, ap, am = bp[:, 2:4], bm[:, 2:4], bp[:, 4], bm[:, 4]
        return float(CV * np.sum((vp - vm) * (vp + vm)) + CA * np.sum((ap - am) * (ap + am)))

    def final_of(p):
        def run(h):
            scenes = make(gpu_lib, seeds)
            apply_pose(gpu_lib, scenes, *p, h)
            batch = gpu_lib.cpGpuBatchNew()
            for sc in scenes:
                gpu_lib.cpGpuBatchAddSpace(batch, sc.space)
            assert gpu_lib.cpGpuBatchStep(batch, DT, STEPS, 0) == 0
            b = np.concatenate([sc.bodies() for sc in scenes])
            gpu_lib.cpGpuBatchFree(batch)
            for sc in scenes:
                sc.free()
            return b
        return run

    smooth, resolved, bad = 0, 0, []
    for kind, w, i, c in params:
        k = w * SIZE + i
        adj = g[kind][2 * k + c] if kind in ("p", "v") else g[kind][k]
        fds = central_difference(final_of((kind, w, i, c)), t, extra)
        kink, res, ok, u = fd_verdict(adj, fds)
        print("%s w%d i%d c%d adjoint %+.10e fd %+.10e %+.10e %+.10e u %.1e%s" % (
            kind, w, i, c, adj, *fds, u / max(abs(fds[1]), 1e-300), "  (contact event)" if kink else ""))
        smooth += not kink
        resolved += res
        if not ok:
            bad.append((kind, w, i, c, adj, fds))
    assert smooth >= 0.7 * len(params), smooth
    assert resolved >= 4, resolved
    assert not bad, bad

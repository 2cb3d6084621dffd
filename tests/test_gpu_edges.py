"""Edge cases of the drop-in, built through the C API in both libraries
(the GPU library and the CPU oracle) and compared: spaces with nothing to
collide, kinematic bodies driving dynamic ones, one iteration, a zero
time step, far-from-origin coordinates, and a batch that mixes empty,
static-only and populated worlds.  Reference-order results must agree to
1e-12 relative per component."""
import numpy as np
import pytest

from chipmunk2d_gb300 import Scene, cpVect

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def v(x, y):
    return cpVect(x, y)


class World:
    """A small scene built through the public API of one library."""

    def __init__(self, lib, kind, offset=(0.0, 0.0), iterations=10):
        self.lib, self.bodies, self.shapes = lib, [], []
        sp = self.space = lib.cpSpaceNew()
        lib.cpSpaceSetGravity(sp, v(0, -100))
        lib.cpSpaceSetIterations(sp, iterations)
        ox, oy = offset
        if kind in ("static_only", "pile", "kinematic"):
            ground = lib.cpSegmentShapeNew(lib.cpSpaceGetStaticBody(sp), v(ox - 100, oy), v(ox + 100, oy), 0.0)
            lib.cpShapeSetFriction(ground, 1.0)
            lib.cpSpaceAddShape(sp, ground)
            self.shapes.append(ground)
        if kind in ("pile", "kinematic"):
            for i in range(12):
                r = 1.0 + 0.1 * (i % 4)
                b = lib.cpSpaceAddBody(sp, lib.cpBodyNew(1.0, lib.cpMomentForCircle(1.0, 0.0, r, v(0, 0))))
                lib.cpBodySetPosition(b, v(ox - 8 + 3.1 * (i % 6), oy + 2 + 2.6 * (i // 6)))
                s = lib.cpSpaceAddShape(sp, lib.cpCircleShapeNew(b, r, v(0, 0)))
                lib.cpShapeSetFriction(s, 0.7)
                self.bodies.append(b); self.shapes.append(s)
        if kind == "kinematic":
            k = lib.cpSpaceAddBody(sp, lib.cpBodyNewKinematic())
            lib.cpBodySetPosition(k, v(ox - 20, oy + 3))
            lib.cpBodySetVelocity(k, v(15, 0))
            s = lib.cpSpaceAddShape(sp, lib.cpBoxShapeNew(k, 4, 4, 0.0))
            self.bodies.append(k); self.shapes.append(s)
        if kind == "free_body":
            b = lib.cpSpaceAddBody(sp, lib.cpBodyNew(2.0, 3.0))
            lib.cpBodySetVelocity(b, v(3, 7))
            self.bodies.append(b)

    def state(self):
        out = []
        for b in self.bodies:
            p, vel = self.lib.cpBodyGetPosition(b), self.lib.cpBodyGetVelocity(b)
            out.append([p.x, p.y, vel.x, vel.y, self.lib.cpBodyGetAngle(b), self.lib.cpBodyGetAngularVelocity(b)])
        return np.array(out).reshape(-1, 6)

    def free(self):
        self.lib.cpSpaceFree(self.space)
        for s in self.shapes:
            self.lib.cpShapeFree(s)
        for b in self.bodies:
            self.lib.cpBodyFree(b)


def rel_err(a, b):
    if a.size == 0:
        return 0.0
    scale = np.maximum(np.abs(b).max(axis=0), 1.0)
    return float((np.abs(a - b) / scale).max())


def run_pair(gpu_lib, oracle_lib, kind, steps, dt=1 / 60, **kw):
    """Free runs of the same world in both libraries; the largest error
    over the steps."""
    g, o = World(gpu_lib, kind, **kw), World(oracle_lib, kind, **kw)
    try:
        worst = 0.0
        for _ in range(steps):
            gpu_lib.cpSpaceStep(g.space, dt)
            oracle_lib.cpSpaceStep(o.space, dt)
            assert gpu_lib.cpGpuGetLastError() == 0, gpu_lib.cpGpuGetLastErrorString().decode()
            worst = max(worst, rel_err(g.state(), o.state()))
        return worst, g.state(), o.state()
    finally:
        g.free(); o.free()


@pytest.mark.parametrize("kind", ["empty", "static_only", "free_body"])
def test_spaces_with_nothing_to_collide(gpu_lib, oracle_lib, kind):
    worst, gs, os_ = run_pair(gpu_lib, oracle_lib, kind, 30)
    assert gs.shape == os_.shape
    assert worst <= RTOL, worst


def test_kinematic_body_drives_a_pile(gpu_lib, oracle_lib):
    worst, gs, _ = run_pair(gpu_lib, oracle_lib, "kinematic", 60)
    assert worst <= 1e-9, worst                 # a free run: sin/cos last-bit drift only
    assert gs[-1, 0] > -20 + 15 * 60 / 60 - 1e-9   # the kinematic box moved at its velocity


def test_one_iteration_and_far_coordinates(gpu_lib, oracle_lib):
    """One solver iteration (the fewest the API accepts: 0 is a hard
    assertion, as in the reference) and a pile a million units from the
    origin."""
    worst, _, _ = run_pair(gpu_lib, oracle_lib, "pile", 40, iterations=1)
    assert worst <= 1e-9, worst
    worst, _, _ = run_pair(gpu_lib, oracle_lib, "pile", 40, offset=(1.0e6, -3.0e5))
    assert worst <= 1e-9, worst


def test_zero_time_step_changes_nothing(gpu_lib):
    w = World(gpu_lib, "pile")
    try:
        for _ in range(5):
            gpu_lib.cpSpaceStep(w.space, 1 / 60)
        before = w.state()
        gpu_lib.cpSpaceStep(w.space, 0.0)
        np.testing.assert_array_equal(w.state(), before)
    finally:
        w.free()


def test_batch_mixing_empty_and_populated_worlds(gpu_lib):
    """Worlds with no bodies, with only static shapes and with piles, in
    one batch: each populated world ends bit-identical to stepping it
    alone."""
    kinds = ["empty", "pile", "static_only", "kinematic", "empty", "pile"]
    batch_worlds = [World(gpu_lib, k, offset=(10.0 * i, 0.0)) for i, k in enumerate(kinds)]
    alone = [World(gpu_lib, k, offset=(10.0 * i, 0.0)) for i, k in enumerate(kinds)]
    batch = gpu_lib.cpGpuBatchNew()
    try:
        for w in batch_worlds:
            assert gpu_lib.cpGpuBatchAddSpace(batch, w.space) >= 0
        assert gpu_lib.cpGpuBatchStep(batch, 1 / 60, 50, 0) == 0, gpu_lib.cpGpuGetLastErrorString().decode()
        for w in alone:
            for _ in range(50):
                gpu_lib.cpSpaceStep(w.space, 1 / 60)
        assert gpu_lib.cpGpuGetLastError() == 0
        for a, b in zip(batch_worlds, alone):
            np.testing.assert_array_equal(a.state(), b.state())
    finally:
        gpu_lib.cpGpuBatchFree(batch)
        for w in batch_worlds + alone:
            w.free()

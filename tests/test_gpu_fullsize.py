"""Full-size parity of the exact-order mode against the oracle.

The benchmark spaces at their own sizes: the 20,000-circle space and the
40,000-body mixed space (30,000 shapes of every kind, 500 pivot chains of
20), and the batch of 4096 uneven tumble worlds (~500,000 bodies).  These
are the sizes at which the per-world tables (pairs, nodes, candidates,
arbiters) and the whole-grid solve are sized by the large cases rather
than by the scaled-down parity scenes.

Every step is teacher-forced (bodies and warm-start impulses copied from
the oracle, as in test_gpu_parity.py), and the arbiter lists must agree
exactly at every step, since the impulse copy fails on any difference.
The state comparison at 1e-12 runs over the first steps and over a window
later in the run, where the circles have piled up (about 33,000 arbiters
at step 295, against about 1,300 in the first 30 steps).
"""
import ctypes

import numpy as np
import pytest

from chipmunk2d_gb300 import Scene
from test_gpu_parity import RTOL, check_gpu_error, compare_step, force

pytestmark = pytest.mark.gpu

# name, scene config, size, iterations' dt, compared step ranges
FULL = [
    ("circles20k", 2, 20000, 1 / 60, [(0, 30), (290, 310)]),
    ("mixed40k", 3, 30000, 1 / 60, [(0, 30), (90, 100)]),
]


@pytest.mark.parametrize("name,cfg,size,dt,windows", FULL, ids=[c[0] for c in FULL])
def test_full_size_teacher_forced(gpu_lib, oracle_lib, name, cfg, size, dt, windows):
    g = Scene(gpu_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    last = max(b for _, b in windows)
    worst, arbs_seen, compared = [0.0, 0.0, 0.0], 0, 0
    try:
        for s in range(last):
            force(g, o)
            g.step(dt)
            o.step(dt)
            if any(a <= s < b for a, b in windows):
                check_gpu_error(gpu_lib)
                errs = compare_step(g, o, s)
                worst = [max(x, y) for x, y in zip(worst, errs)]
                assert max(errs) <= RTOL, "%s step %d: body %.3g arbiter %.3g joint %.3g" % ((name, s) + errs)
                compared += 1
                arbs_seen = max(arbs_seen, len(o.arbiters()))
        check_gpu_error(gpu_lib)
    finally:
        g.free()
        o.free()
    assert compared == sum(b - a for a, b in windows)
    print("%s: %d steps compared, up to %d arbiters, worst rel err bodies %.3g arbiters %.3g joints %.3g"
          % (name, compared, arbs_seen, *worst))


def test_full_batch_of_4096_worlds(gpu_lib, oracle_lib):
    """All 4096 worlds of the batch workload at their own sizes (8 to 512
    bodies, log-uniform), stepped together for 20 teacher-forced steps,
    against the oracle stepping each world alone."""
    n = 4096
    sizes = (ctypes.c_int * n)()
    gpu_lib.cpx_batch_sizes(n, 3, ctypes.cast(sizes, ctypes.c_void_p))
    gs = [Scene(gpu_lib, 4, sizes[i], seed=1000 + i) for i in range(n)]
    os_ = [Scene(oracle_lib, 4, sizes[i], seed=1000 + i) for i in range(n)]
    batch = gpu_lib.cpGpuBatchNew()
    try:
        for g in gs:
            assert gpu_lib.cpGpuBatchAddSpace(batch, g.space) >= 0
        worst = 0.0
        for s in range(20):
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
        print("4096 worlds, %d bodies: worst rel err %.3g" % (sum(sizes[i] for i in range(n)), worst))
    finally:
        gpu_lib.cpGpuBatchFree(batch)
        for g in gs:
            g.free()
        for o in os_:
            o.free()

"""The spatial hash (cpSpaceUseSpatialHash, src/cpSpaceHash.c) as the
broadphase of seeded workloads.

The switch is made after the workload is built, so every shape is copied
from the trees into the hashes in the reference's order.  On the CPU the
oracle is pinned to the reference bit for bit after every step; on the GPU
each step is teacher-forced from the oracle and compared as in
test_gpu_parity.py (arbiter pairs and solve order exact).  Seeded queries
run on the hash at the end, visit orders included.
"""
import ctypes

import numpy as np
import pytest

from chipmunk2d_gb300 import Scene
from test_gpu_parity import check_gpu_error, compare_step, force

# (workload, size, steps, cell size, cells)
CASES = [(1, 14, 200, 40.0, 1000), (2, 1500, 120, 4.0, 4000), (3, 900, 100, 8.0, 2000), (6, 200, 150, 6.0, 2000)]
IDS = ["pyramid", "circles", "mixed", "joints"]


def use_hash(lib, sc, dim, cells):
    lib.cpSpaceUseSpatialHash.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int]
    lib.cpSpaceUseSpatialHash(sc.space, dim, cells)


@pytest.mark.parametrize("cfg,size,steps,dim,cells", CASES, ids=IDS)
def test_oracle_bit_exact_on_the_spatial_hash(ref_lib, oracle_lib, cfg, size, steps, dim, cells):
    r = Scene(ref_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    try:
        use_hash(ref_lib, r, dim, cells)
        use_hash(oracle_lib, o, dim, cells)
        for s in range(steps):
            r.step(1 / 60)
            o.step(1 / 60)
            np.testing.assert_array_equal(o.bodies(), r.bodies(), err_msg="bodies, step %d" % s)
            np.testing.assert_array_equal(o.arbiters(), r.arbiters(), err_msg="arbiters, step %d" % s)
            np.testing.assert_array_equal(o.constraints(), r.constraints(), err_msg="joints, step %d" % s)
        np.testing.assert_array_equal(o.queries(5, 48), r.queries(5, 48))
    finally:
        r.free()
        o.free()


@pytest.mark.gpu
@pytest.mark.parametrize("cfg,size,steps,dim,cells", CASES, ids=IDS)
def test_teacher_forced_on_the_spatial_hash(gpu_lib, oracle_lib, cfg, size, steps, dim, cells):
    g = Scene(gpu_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    try:
        use_hash(gpu_lib, g, dim, cells)
        use_hash(oracle_lib, o, dim, cells)
        worst = 0.0
        for s in range(steps):
            if s > 0:
                force(g, o)
            g.step(1 / 60)
            o.step(1 / 60)
            check_gpu_error(gpu_lib)
            eb, ea, _ = compare_step(g, o, s)
            worst = max(worst, eb, ea)
        qg, qo = g.queries(5, 48), o.queries(5, 48)
        check_gpu_error(gpu_lib)
        assert qg.shape == qo.shape
        np.testing.assert_array_equal(qg[:, 0], qo[:, 0])
        np.testing.assert_allclose(qg, qo, rtol=1e-9, atol=1e-9)
        print("workload %d on the spatial hash: worst rel err %.3g" % (cfg, worst))
    finally:
        g.free()
        o.free()

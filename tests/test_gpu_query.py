"""Spatial queries on the device (cpSpacePointQuery, cpSpacePointQueryNearest,
cpSpaceSegmentQuery, cpSpaceSegmentQueryFirst, cpSpaceBBQuery,
cpShapePointQuery, cpShapeSegmentQuery) against the oracle.

The scenes' query harness (scenes.c, cpx_scene_queries) records every
callback in call order and every result.  In the exact-order mode the GPU
walks the same trees in the same order, so the records must agree row for
row: query, kind and shape exactly, the geometry within 1e-12 (scaled by
the magnitude of each column; teacher-forced steps leave the last bit of
sin/cos in the body transforms).  In the coloured mode every shape is
tested in slot order, so each query's set of hits must agree (segment
queries there find every shape the thick segment touches).
"""
import ctypes

import numpy as np
import pytest

from chipmunk2d_gb300 import Scene
from test_gpu_parity import check_gpu_error, force

pytestmark = pytest.mark.gpu

RTOL = 1e-12
CASES = [(1, 14, 40), (2, 1500, 120), (3, 1200, 60), (6, 200, 80), (7, 40, 80)]


def same_records(g, o, what):
    assert g.shape == o.shape, "%s: %d records on the GPU, %d in the oracle" % (what, len(g), len(o))
    np.testing.assert_array_equal(g[:, :3], o[:, :3], err_msg="%s: query, kind, shape" % what)
    if len(o):
        scale = np.maximum(np.abs(o[:, 3:]).max(axis=0), 1.0)
        err = float((np.abs(g[:, 3:] - o[:, 3:]) / scale).max())
        assert err <= RTOL, "%s: geometry differs by %.3g" % (what, err)


def hit_sets(rec):
    """Per (query, kind): the set of shapes hit (the multi-hit kinds) or the
    single result's shape."""
    out = {}
    for row in rec:
        out.setdefault((int(row[0]), int(row[1])), set()).add(int(row[2]))
    return out


@pytest.mark.parametrize("cfg,size,steps", CASES, ids=["pyramid", "circles", "mixed", "joints", "machines"])
def test_queries_match_oracle_in_tree_order(gpu_lib, oracle_lib, cfg, size, steps):
    g = Scene(gpu_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    try:
        # before the first step: the query builds the device set
        same_records(g.queries(1, 140), o.queries(1, 140), "before the first step")
        check_gpu_error(gpu_lib)
        for _ in range(steps):
            force(g, o)
            g.step(1 / 60)
            o.step(1 / 60)
        qg, qo = g.queries(2, 700), o.queries(2, 700)
        check_gpu_error(gpu_lib)
        assert len(qo) > 100
        same_records(qg, qo, "after %d steps" % steps)
        # edits between steps are indexed before the query runs
        if cfg in (1, 3, 6):
            assert g.edit(0, 7) == o.edit(0, 7)
            same_records(g.queries(3, 140), o.queries(3, 140), "after edits")
            check_gpu_error(gpu_lib)
    finally:
        g.free()
        o.free()


@pytest.mark.parametrize("cfg,size", [(2, 1500), (3, 1200), (6, 200)], ids=["circles", "mixed", "joints"])
def test_coloured_mode_queries_find_the_same_shapes(gpu_lib, cfg, size):
    """The coloured mode tests every shape instead of walking the dynamic
    tree; on the same state it must find the same shapes as the tree walk."""
    g = Scene(gpu_lib, cfg, size)
    try:
        for _ in range(60):
            g.step(1 / 60)
        tree = g.queries(5, 700)
        gpu_lib.cpGpuSetSolverMode(g.space, 1)
        brute = g.queries(5, 700)
        gpu_lib.cpGpuSetSolverMode(g.space, 0)
        check_gpu_error(gpu_lib)
        ts, bs = hit_sets(tree), hit_sets(brute)
        # point and box queries: the same shapes; segment queries: the
        # tree's hits and any shape the thick segment grazes outside the
        # boxes the tree tests
        for key in set(ts) | set(bs):
            if key[1] in (0, 4):
                assert ts.get(key, set()) == bs.get(key, set()), key
            elif key[1] == 2:
                assert ts.get(key, set()) <= bs.get(key, set()), key
        for k in (1, 5, 6):
            np.testing.assert_array_equal(tree[tree[:, 1] == k], brute[brute[:, 1] == k])
        # first hit: never later than the tree's
        ft, fb = tree[tree[:, 1] == 3], brute[brute[:, 1] == 3]
        assert len(ft) == len(fb) and (fb[:, 5] <= ft[:, 5]).all()
    finally:
        g.free()


class Filter(ctypes.Structure):
    _fields_ = [("group", ctypes.c_size_t), ("categories", ctypes.c_uint), ("mask", ctypes.c_uint)]


INFO = np.dtype([("shape", np.uint64), ("px", np.float64), ("py", np.float64),
                 ("a", np.float64), ("b", np.float64), ("c", np.float64)])


def test_batched_raycasts_match_single_queries(gpu_lib, oracle_lib):
    """cpGpuSpaceSegmentQueryFirstBatch and cpGpuSpacePointQueryNearestBatch
    answer many queries in one launch; each answer equals the single query's
    (cpSpaceSegmentQueryFirst, cpSpacePointQueryNearest) on the oracle."""
    cfg, size = 2, 1500
    g = Scene(gpu_lib, cfg, size)
    o = Scene(oracle_lib, cfg, size)
    try:
        for _ in range(80):
            force(g, o)
            g.step(1 / 60)
            o.step(1 / 60)
        rng = np.random.default_rng(7)
        n = 4096
        pos = o.bodies()[:, 0:2]
        starts = np.ascontiguousarray(pos[rng.integers(0, len(pos), n)] + rng.normal(0, 3, size=(n, 2)))
        ends = np.ascontiguousarray(starts + rng.normal(0, 60, size=(n, 2)))
        flt = Filter(0, 0xFFFFFFFF, 0xFFFFFFFF)
        seg = np.zeros(n, dtype=INFO)
        fn = gpu_lib.cpGpuSpaceSegmentQueryFirstBatch
        fn.restype = ctypes.c_int
        fn.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_double, Filter, ctypes.c_void_p]
        assert fn(g.space, n, starts.ctypes.data, ends.ctypes.data, 0.5, flt, seg.ctypes.data) == 0
        near = np.zeros(n, dtype=INFO)
        fn2 = gpu_lib.cpGpuSpacePointQueryNearestBatch
        fn2.restype = ctypes.c_int
        fn2.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_double, Filter, ctypes.c_void_p]
        assert fn2(g.space, n, starts.ctypes.data, 10.0, flt, near.ctypes.data) == 0
        check_gpu_error(gpu_lib)
        hits = int((seg["shape"] != 0).sum())
        assert hits > n // 8
        # the oracle's single queries, by shape index through the user data
        oracle_lib.cpShapeGetUserData.restype = ctypes.c_void_p
        oracle_lib.cpShapeGetUserData.argtypes = [ctypes.c_void_p]
        gpu_lib.cpShapeGetUserData.restype = ctypes.c_void_p
        gpu_lib.cpShapeGetUserData.argtypes = [ctypes.c_void_p]
        o.queries(0, 1)     # sets every shape's user data to its index + 1
        g.queries(0, 1)
        ofirst = oracle_lib.cpSpaceSegmentQueryFirst
        ofirst.restype = ctypes.c_void_p
        onear = oracle_lib.cpSpacePointQueryNearest
        onear.restype = ctypes.c_void_p
        from chipmunk2d_gb300 import cpVect
        ofirst.argtypes = [ctypes.c_void_p, cpVect, cpVect, ctypes.c_double, Filter, ctypes.c_void_p]
        onear.argtypes = [ctypes.c_void_p, cpVect, ctypes.c_double, Filter, ctypes.c_void_p]
        one = np.zeros(1, dtype=INFO)
        for i in range(0, n, 7):
            s = ofirst(o.space, cpVect(*starts[i]), cpVect(*ends[i]), 0.5, flt, one.ctypes.data)
            gi = gpu_lib.cpShapeGetUserData(int(seg["shape"][i])) if seg["shape"][i] else 0
            oi = oracle_lib.cpShapeGetUserData(s) if s else 0
            assert (gi or 0) == (oi or 0), "ray %d" % i
            for f in ("px", "py", "a", "b", "c"):
                assert abs(seg[f][i] - one[f][0]) <= RTOL * max(1.0, abs(one[f][0])), (i, f)
            s = onear(o.space, cpVect(*starts[i]), 10.0, flt, one.ctypes.data)
            gi = gpu_lib.cpShapeGetUserData(int(near["shape"][i])) if near["shape"][i] else 0
            oi = oracle_lib.cpShapeGetUserData(s) if s else 0
            assert (gi or 0) == (oi or 0), "point %d" % i
            for f in ("px", "py", "a", "b", "c"):
                assert abs(near[f][i] - one[f][0]) <= RTOL * max(1.0, abs(one[f][0])), (i, f)
    finally:
        g.free()
        o.free()

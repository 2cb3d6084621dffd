"""Saved states (cpGpuSpaceSaveState / cpGpuSpaceRestoreState): a restored
space repeats its steps from the save bit for bit, in both solver modes,
and restoring after an object edit is refused."""
import ctypes

import numpy as np
import pytest

from chipmunk2d_gb300 import Scene, cpVect
from test_gpu_parity import check_gpu_error

pytestmark = pytest.mark.gpu


def bind_state(lib):
    lib.cpGpuSpaceSaveState.restype = ctypes.c_void_p
    lib.cpGpuSpaceSaveState.argtypes = [ctypes.c_void_p]
    lib.cpGpuSpaceRestoreState.restype = ctypes.c_int
    lib.cpGpuSpaceRestoreState.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
    lib.cpGpuSpaceStateFree.restype = None
    lib.cpGpuSpaceStateFree.argtypes = [ctypes.c_void_p]


def canon(rec, mode):
    """The coloured mode appends arbiters to its solve list with atomics:
    the list's order is free (units of one colour commute), so its records
    are compared sorted by shape pair."""
    if mode == 1 and rec.ndim == 2 and rec.shape[1] == 34:
        return rec[np.lexsort((rec[:, 1], rec[:, 0]))]
    return rec


@pytest.mark.parametrize("cfg,size,mode", [(2, 1500, 0), (2, 1500, 1), (6, 200, 0), (7, 40, 0), (3, 1200, 1)],
                         ids=["circles-ordered", "circles-coloured", "joints", "machines", "mixed-coloured"])
def test_restored_state_repeats_the_steps(gpu_lib, cfg, size, mode):
    bind_state(gpu_lib)
    g = Scene(gpu_lib, cfg, size)
    gpu_lib.cpGpuSetSolverMode(g.space, mode)
    st = None
    try:
        for _ in range(40):
            g.step(1 / 60)
        saved = (g.bodies(), g.arbiters(), g.constraints())
        st = gpu_lib.cpGpuSpaceSaveState(g.space)
        assert st, gpu_lib.cpGpuGetLastErrorString().decode()
        for _ in range(50):
            g.step(1 / 60)
        first = (g.bodies(), g.arbiters(), g.constraints(), g.public())
        assert gpu_lib.cpGpuSpaceRestoreState(g.space, st) == 0
        back = (g.bodies(), g.arbiters(), g.constraints())
        for a, b in zip(back, saved):
            np.testing.assert_array_equal(canon(a, mode), canon(b, mode))
        for _ in range(50):
            g.step(1 / 60)
        again = (g.bodies(), g.arbiters(), g.constraints(), g.public())
        check_gpu_error(gpu_lib)
        for a, b in zip(again, first):
            np.testing.assert_array_equal(canon(a, mode), canon(b, mode))
    finally:
        if st:
            gpu_lib.cpGpuSpaceStateFree(st)
        g.free()


def test_restore_after_an_edit_is_refused(gpu_lib):
    bind_state(gpu_lib)
    g = Scene(gpu_lib, 1, 14)
    try:
        for _ in range(10):
            g.step(1 / 60)
        st = gpu_lib.cpGpuSpaceSaveState(g.space)
        assert st
        g.step(1 / 60)
        gpu_lib.cpBodySetVelocity(gpu_lib.cpx_scene_body(g.h, 3), cpVect(1.0, 2.0))
        assert gpu_lib.cpGpuSpaceRestoreState(g.space, st) == 3          # CP_GPU_ERR_UNSUPPORTED
        assert gpu_lib.cpGpuGetLastError() == 3
        gpu_lib.cpGpuSpaceStateFree(st)
        # a save after the edit restores
        st = gpu_lib.cpGpuSpaceSaveState(g.space)
        g.step(1 / 60)
        assert gpu_lib.cpGpuSpaceRestoreState(g.space, st) == 0
        gpu_lib.cpGpuSpaceStateFree(st)
        # objects removed since the save
        st = gpu_lib.cpGpuSpaceSaveState(g.space)
        assert g.edit(0, 7) >= 0
        assert gpu_lib.cpGpuSpaceRestoreState(g.space, st) == 3
        gpu_lib.cpGpuGetLastError()
        gpu_lib.cpGpuSpaceStateFree(st)
    finally:
        g.free()


@pytest.mark.parametrize("mode", [0, 1], ids=["ordered", "coloured"])
def test_bulk_body_states_equal_the_getters(gpu_lib, mode):
    """cpGpuSpaceGetBodyStates returns, in one read, exactly what the
    per-body getters return: before the first step (host state), after
    steps (gathered on the device) and after a host edit."""
    gpu_lib.cpGpuSpaceGetBodyStates.restype = ctypes.c_int
    gpu_lib.cpGpuSpaceGetBodyStates.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int]
    g = Scene(gpu_lib, 3, 600)
    gpu_lib.cpGpuSetSolverMode(g.space, mode)
    try:
        n = g.nbodies
        for steps in (0, 1, 30):
            for _ in range(steps):
                g.step(1 / 60)
            bulk = np.zeros(8 * n)
            assert gpu_lib.cpGpuSpaceGetBodyStates(g.space, bulk.ctypes.data, n) == n
            np.testing.assert_array_equal(bulk.reshape(n, 8), g.public())
        gpu_lib.cpBodySetVelocity(gpu_lib.cpx_scene_body(g.h, 5), cpVect(3.0, -4.0))
        bulk = np.zeros(8 * n)
        assert gpu_lib.cpGpuSpaceGetBodyStates(g.space, bulk.ctypes.data, n) == n
        np.testing.assert_array_equal(bulk.reshape(n, 8), g.public())
        assert bulk[8 * 5 + 2] == 3.0 and bulk[8 * 5 + 3] == -4.0
        check_gpu_error(gpu_lib)
    finally:
        g.free()

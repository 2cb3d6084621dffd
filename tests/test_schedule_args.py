"""Argument checks of the schedule entry points run on the host before any
CUDA call, so they are tested here without a GPU.  levelStart receives
levelStart[0] = 0 even for an empty unit sequence: a NULL levelStart must
be refused for every nunits, never handed to the kernel."""
import ctypes
import os

import pytest

from chipmunk2d_gb300._lib import LIB_PATH, bind

CP_GPU_ERR_ARGUMENT = 6
NZ = ctypes.c_void_p(8)   # a non-null pointer the checks never dereference


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB_PATH):
        from chipmunk2d_gb300.build import build
        build()
    return bind(LIB_PATH, gpu=True)


@pytest.mark.parametrize("fn", ["cpGpuSolveSchedule", "cpGpuSolveScheduleNoAlloc"])
def test_null_level_start_is_refused_for_empty_input(lib, fn):
    assert getattr(lib, fn)(None, None, 0, 0, None, None, NZ, None) == CP_GPU_ERR_ARGUMENT
    assert getattr(lib, fn)(None, None, 0, 5, None, NZ, NZ, None) == CP_GPU_ERR_ARGUMENT


@pytest.mark.parametrize("fn", ["cpGpuSolveSchedule", "cpGpuSolveScheduleNoAlloc"])
def test_missing_arrays_are_refused(lib, fn):
    f = getattr(lib, fn)
    assert f(None, NZ, 3, 4, NZ, NZ, NZ, None) == CP_GPU_ERR_ARGUMENT     # bodyA
    assert f(NZ, None, 3, 4, NZ, NZ, NZ, None) == CP_GPU_ERR_ARGUMENT     # bodyB
    assert f(NZ, NZ, 3, 4, NZ, None, NZ, None) == CP_GPU_ERR_ARGUMENT     # order
    assert f(NZ, NZ, 3, 4, NZ, NZ, None, None) == CP_GPU_ERR_ARGUMENT     # nlevels
    assert f(NZ, NZ, -1, 4, NZ, NZ, NZ, None) == CP_GPU_ERR_ARGUMENT
    assert f(NZ, NZ, 3, -1, NZ, NZ, NZ, None) == CP_GPU_ERR_ARGUMENT


def test_no_alloc_rejects_sizes_beyond_its_scratch_on_the_host(lib):
    f = lib.cpGpuSolveScheduleNoAlloc
    assert f(NZ, NZ, (1 << 20) + 1, 4, NZ, NZ, NZ, None) == CP_GPU_ERR_ARGUMENT
    assert f(NZ, NZ, 4, (1 << 20) + 1, NZ, NZ, NZ, None) == CP_GPU_ERR_ARGUMENT

"""cpGpuSolveScheduleNoAlloc, the allocation-free schedule entry point.

It exists for callers that cannot allocate device memory when they need a
schedule (a frame loop with a fixed time budget, or a host application
whose memory manager owns all device memory).  This test calls it through
the C ABI and checks its output against cpGpuSolveSchedule, which allocates
its scratch, on two calls in a row with different sizes (the second call
reuses the fixed scratch the first one left behind).  The outputs are
integer schedules, so they must be identical.  It also checks that the
call leaves the device's free memory unchanged and that inputs beyond the
fixed maximum are refused.  This file is collected last so that a run that
stops at the first failure has already run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(lib, fn, a, b, nbodies):
    torch = pytest.importorskip("torch")
    n = len(a)
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    start = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
    order = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    nlev = torch.full((1,), -7, dtype=torch.int32, device="cuda")
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream().cuda_stream
    rc = getattr(lib, fn)(ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(db.data_ptr()), n, nbodies,
                          ctypes.c_void_p(start.data_ptr()), ctypes.c_void_p(order.data_ptr()),
                          ctypes.c_void_p(nlev.data_ptr()), ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    assert rc == 0
    L = int(nlev.item())
    return L, start.cpu().numpy()[:L + 1], order.cpu().numpy()[:n]


def test_no_alloc_schedule_matches_allocating_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(11)
    # first call: many units on few bodies (deep schedule);
    # second call: fewer units on more bodies, after the first left its scratch behind
    for nunits, nbodies in ((6000, 400), (2500, 3000)):
        a = rng.integers(-1, nbodies, nunits).astype(np.int32)
        b = rng.integers(-1, nbodies, nunits).astype(np.int32)
        L0, s0, o0 = _run(gpu_lib, "cpGpuSolveSchedule", a, b, nbodies)
        free_before = torch.cuda.mem_get_info()[0]
        L1, s1, o1 = _run(gpu_lib, "cpGpuSolveScheduleNoAlloc", a, b, nbodies)
        free_after = torch.cuda.mem_get_info()[0]
        assert L1 == L0
        np.testing.assert_array_equal(s1, s0)
        np.testing.assert_array_equal(o1, o0)
        assert free_after >= free_before


def test_no_alloc_schedule_rejects_sizes_beyond_its_scratch(gpu_lib):
    assert gpu_lib.cpGpuSolveScheduleNoAlloc(ctypes.c_void_p(8), ctypes.c_void_p(8), (1 << 20) + 1, 4,
                                             ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8), None) != 0
    assert gpu_lib.cpGpuSolveScheduleNoAlloc(ctypes.c_void_p(8), ctypes.c_void_p(8), 4, (1 << 20) + 1,
                                             ctypes.c_void_p(8), ctypes.c_void_p(8), ctypes.c_void_p(8), None) != 0

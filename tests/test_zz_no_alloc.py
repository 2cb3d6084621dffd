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


_FRESH = r'''
import ctypes, sys
import numpy as np
import torch
sys.path.insert(0, sys.argv[1])
from chipmunk2d_gb300 import load_gpu_library
lib = load_gpu_library()
vp = ctypes.c_void_p
# unrelated CUDA work first: the context exists, this library's code is not loaded yet
x = torch.arange(1000, device="cuda", dtype=torch.float64)
assert float((x * 2).sum().item()) == 999000.0
rng = np.random.default_rng(5)
calls = []
for nunits, nbodies in ((4000, 250), (1500, 2000)):
    a = torch.from_numpy(rng.integers(-1, nbodies, nunits).astype(np.int32)).cuda()
    b = torch.from_numpy(rng.integers(-1, nbodies, nunits).astype(np.int32)).cuda()
    outs = [(torch.full((nunits + 1,), -7, dtype=torch.int32, device="cuda"),
             torch.full((nunits,), -7, dtype=torch.int32, device="cuda"),
             torch.full((1,), -7, dtype=torch.int32, device="cuda")) for _ in range(2)]
    calls.append((nunits, nbodies, a, b, outs))
ls = torch.full((1,), -7, dtype=torch.int32, device="cuda")
nl = torch.full((1,), -7, dtype=torch.int32, device="cuda")
stream = torch.cuda.current_stream().cuda_stream
torch.cuda.synchronize()
# the documented start-up call: an empty sequence (this is the set-up)
assert lib.cpGpuSolveScheduleNoAlloc(None, None, 0, 0, vp(ls.data_ptr()), None, vp(nl.data_ptr()), vp(stream)) == 0
torch.cuda.synchronize()
assert int(ls.item()) == 0 and int(nl.item()) == 0
free0 = torch.cuda.mem_get_info()[0]
for nunits, nbodies, a, b, outs in calls:
    s, o, n = outs[0]
    rc = lib.cpGpuSolveScheduleNoAlloc(vp(a.data_ptr()), vp(b.data_ptr()), nunits, nbodies,
                                       vp(s.data_ptr()), vp(o.data_ptr()), vp(n.data_ptr()), vp(stream))
    torch.cuda.synchronize()
    assert rc == 0
free1 = torch.cuda.mem_get_info()[0]
assert free1 >= free0, (free0, free1)
# the allocating entry point on the same inputs, afterwards
for nunits, nbodies, a, b, outs in calls:
    s, o, n = outs[1]
    rc = lib.cpGpuSolveSchedule(vp(a.data_ptr()), vp(b.data_ptr()), nunits, nbodies,
                                vp(s.data_ptr()), vp(o.data_ptr()), vp(n.data_ptr()), vp(stream))
    torch.cuda.synchronize()
    assert rc == 0
    L = int(outs[0][2].item())
    assert L == int(n.item()) and L > 0
    assert torch.equal(outs[0][0][:L + 1], s[:L + 1]) and torch.equal(outs[0][1], o)
print("fresh-process no-alloc ok", free0, free1)
'''


def test_no_alloc_first_in_a_fresh_process():
    """In a new process whose only earlier CUDA work is unrelated to this
    library, the documented start-up call (an empty sequence) does the
    one-time set-up; after it, two calls leave the device's free memory
    unchanged, and their schedules equal the allocating entry point's."""
    import os
    import subprocess
    import sys
    pytest.importorskip("torch")
    repo = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    r = subprocess.run([sys.executable, "-c", _FRESH, repo], stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-3000:]
    assert "fresh-process no-alloc ok" in r.stdout

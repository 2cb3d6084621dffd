"""cpGpuSolveSchedule: the exact-order level schedule of a sweep, checked
against a direct restatement of the recurrence and for the two properties
that make the level-parallel sweep equal the serial one."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def reference_levels(a, b, nbodies):
    last = np.zeros(nbodies, dtype=np.int64)
    lvl = np.zeros(len(a), dtype=np.int64)
    for u in range(len(a)):
        l = 0
        for x in (a[u], b[u]):
            if 0 <= x < nbodies:
                l = max(l, last[x])
        lvl[u] = l
        for x in (a[u], b[u]):
            if 0 <= x < nbodies:
                last[x] = l + 1
    return lvl


def random_sweep(rng, nunits, nbodies):
    a = rng.integers(-1, nbodies, nunits).astype(np.int32)
    b = rng.integers(-1, nbodies, nunits).astype(np.int32)
    return a, b


def run_schedule(lib, fn, a, b, nbodies):
    torch = pytest.importorskip("torch")
    n = len(a)
    da = torch.from_numpy(a).cuda()
    db = torch.from_numpy(b).cuda()
    start = torch.full((n + 1,), -7, dtype=torch.int32, device="cuda")
    order = torch.full((max(n, 1),), -7, dtype=torch.int32, device="cuda")
    nlev = torch.zeros(1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    rc = getattr(lib, fn)(ctypes.c_void_p(da.data_ptr()), ctypes.c_void_p(db.data_ptr()), n, nbodies,
                          ctypes.c_void_p(start.data_ptr()), ctypes.c_void_p(order.data_ptr()),
                          ctypes.c_void_p(nlev.data_ptr()), ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    assert rc == 0
    L = int(nlev.item())
    return start.cpu().numpy()[:L + 1], order.cpu().numpy()[:n], L


def check_schedule(a, b, nbodies, start, order, L):
    lvl = reference_levels(a, b, nbodies)
    n = len(a)
    assert L == (int(lvl.max()) + 1 if n else 0)
    assert start[0] == 0 and start[L] == n
    expect = np.argsort(lvl, kind="stable")
    np.testing.assert_array_equal(order, expect)
    for l in range(L):
        units = order[start[l]:start[l + 1]]
        touched = [x for u in units for x in {a[u], b[u]} if 0 <= x < nbodies]
        assert len(touched) == len(set(touched)), "level %d reuses a body" % l


@pytest.mark.parametrize("nunits,nbodies,seed", [(0, 5, 0), (1, 1, 1), (200, 20, 2), (5000, 300, 3), (20000, 20000, 4)])
def test_schedule_matches_recurrence(gpu_lib, nunits, nbodies, seed):
    rng = np.random.default_rng(seed)
    a, b = random_sweep(rng, nunits, nbodies)
    start, order, L = run_schedule(gpu_lib, "cpGpuSolveSchedule", a, b, nbodies)
    check_schedule(a, b, nbodies, start, order, L)


def test_schedule_rejects_bad_arguments(gpu_lib):
    assert gpu_lib.cpGpuSolveSchedule(None, None, -1, 4, None, None, None, None) != 0
    # levelStart is written even for an empty sequence, so it is required
    # whatever nunits is (refused on the host, before any launch)
    for fn in ("cpGpuSolveSchedule", "cpGpuSolveScheduleNoAlloc"):
        assert getattr(gpu_lib, fn)(None, None, 0, 0, None, None, ctypes.c_void_p(8), None) != 0

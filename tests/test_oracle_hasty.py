"""The CPU baseline's threaded solver (the oracle's restatement of
cpHastySpace's two-thread solver): it runs, keeps the scene physical, and
hands back to the serial solver.  Its results are not deterministic (the
two threads update shared bodies without synchronisation, as the
reference's do), so they are checked for plausibility only."""
import numpy as np

from chipmunk2d_gb300 import Scene


def test_two_thread_solver_runs_and_stops(oracle_lib):
    sc = Scene(oracle_lib, 1, 14)                    # the 105-box pyramid
    assert oracle_lib.cpx_space_set_hasty(sc.space, 2) == 2
    assert oracle_lib.cpx_space_set_hasty(sc.space, 2) == 2     # already running
    sc.step(1 / 60, 120)
    b = sc.bodies()
    assert np.all(np.isfinite(b))
    # a resting pyramid stays put: no box moved far or fell through the ground
    assert np.abs(b[:, 2:4]).max() < 50.0
    assert b[:, 1].min() > -260.0
    assert oracle_lib.cpx_space_set_hasty(sc.space, 1) == 1     # back to the serial solver
    sc.step(1 / 60, 10)
    sc.free()


def test_space_with_running_workers_frees(oracle_lib):
    sc = Scene(oracle_lib, 2, 500)
    oracle_lib.cpx_space_set_hasty(sc.space, 2)
    sc.step(1 / 60, 5)
    sc.free()                                        # joins the worker thread

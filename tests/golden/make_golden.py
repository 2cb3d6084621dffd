"""Regenerates tests/golden/*.npz from the unmodified reference.

The reference is built from its own sources by oracle/build_ref.sh into
oracle/_ref/libcpref.so; this script drives it through the C API on the
seeded workloads and records the full state (bodies, arbiters in solve
order, joints) at a few checkpoints.  The fixtures travel with the
repository, so the oracle stays pinned where the reference cannot be built.

Usage:  python tests/golden/make_golden.py [fixture names]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from chipmunk2d_gb300 import bind, Scene  # noqa: E402

# (name, workload, size, dt, checkpoints)
FIXTURES = [
    ("pyramid", 1, 14, 1 / 60, [1, 2, 10, 100, 400]),
    ("circles", 2, 600, 1 / 60, [1, 5, 60]),
    ("mixed", 3, 600, 1 / 60, [1, 5, 40]),
    ("tumble", 4, 150, 1 / 60, [1, 5, 60]),
    ("adjoint", 5, 64, 1 / 120, [1, 5, 120]),
    ("joints", 6, 120, 1 / 60, [1, 5, 60, 200]),
    ("machines", 7, 12, 1 / 60, [1, 5, 60, 200]),
]


def main(only=None):
    lib = bind(os.path.join(REPO, "oracle", "_ref", "libcpref.so"))
    for name, cfg, size, dt, checkpoints in FIXTURES:
        if only and name not in only:
            continue
        sc = Scene(lib, cfg, size)
        data = {"config": np.array([cfg, size]), "dt": np.array(dt), "checkpoints": np.array(checkpoints)}
        done = 0
        for c in checkpoints:
            sc.step(dt, c - done)
            done = c
            data["bodies_%d" % c] = sc.bodies()
            data["arbiters_%d" % c] = sc.arbiters()
            data["constraints_%d" % c] = sc.constraints()
            data["public_%d" % c] = sc.public()
            data["impulses_%d" % c] = sc.impulses()
        sc.free()
        path = os.path.join(HERE, name + ".npz")
        np.savez_compressed(path, **data)
        print(path, os.path.getsize(path))


if __name__ == "__main__":
    main(sys.argv[1:])

"""The drop-in library loads without a GPU and exports every entry point that
include/chipmunk_gb300.h declares (no compute calls)."""
import ctypes
import os
import re

import pytest

from chipmunk2d_gb300 import LIB_PATH, HEADER


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = set()
    for m in re.finditer(r"^\s*(?!static|typedef|#|extern\s+const)[A-Za-z_][\w\s\*]*?\b(cp\w+)\s*\(", src, flags=re.M):
        names.add(m.group(1))
    names.add("cpVersionString")
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB_PATH):
        from chipmunk2d_gb300.build import build
        build()
    return ctypes.CDLL(LIB_PATH)


def test_header_declares_the_step_api():
    names = declared_functions()
    for n in ("cpSpaceNew", "cpSpaceAddBody", "cpSpaceAddShape", "cpSpaceAddConstraint",
              "cpSpaceSetIterations", "cpSpaceSetGravity", "cpSpaceStep", "cpArbiterTotalImpulse",
              "cpGpuBatchStep", "cpGpuGetLastError"):
        assert n in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_product_exports_no_test_scaffolding(lib):
    """The seeded workloads and the state-export names live in the
    test-side libcpx_scenes.so, not in the product library."""
    for n in ("cpx_scene_build", "cpx_batch_sizes", "cpx_scene_dump_public", "cpx_dump_bodies"):
        assert not hasattr(lib, n), n

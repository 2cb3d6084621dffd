import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)

ORACLE_SO = os.path.join(REPO, "oracle", "_build", "liboracle.so")
REF_SO = os.path.join(REPO, "oracle", "_ref", "libcpref.so")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libchipmunk_gb300.so")


def _ensure_oracle():
    src = os.path.join(REPO, "oracle", "cp_oracle.c")
    if (not os.path.exists(ORACLE_SO)) or os.path.getmtime(ORACLE_SO) < os.path.getmtime(src):
        subprocess.check_call([os.path.join(REPO, "oracle", "build_oracle.sh")], stdout=subprocess.DEVNULL)
    return ORACLE_SO


@pytest.fixture(scope="session")
def oracle_lib():
    from chipmunk2d_gb300 import bind
    return bind(_ensure_oracle())


@pytest.fixture(scope="session")
def ref_lib():
    """The unmodified reference, when it was built here (oracle/build_ref.sh)."""
    if not os.path.exists(REF_SO):
        pytest.skip("reference library not built on this machine")
    from chipmunk2d_gb300 import bind
    return bind(REF_SO)


@pytest.fixture(scope="session")
def gpu_lib():
    from chipmunk2d_gb300 import load_gpu_library
    return load_gpu_library()

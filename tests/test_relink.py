"""A plain C program (tests/relink_program.c, reference API only) switches
implementations by relinking: it builds against the reference's headers or
this repository's, links against the reference library, the oracle or the
GPU library, and gives the same results.  It adds and removes bodies,
shapes and joints between steps.
"""
import os
import shutil
import subprocess

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PROGRAMS = ["relink_program.c", "relink_program2.c", "relink_program3.c", "relink_program4.c", "relink_program5.c", "relink_program6.c", "relink_program7.c", "relink_program8.c", "relink_program9.c"]
GPU_DIR = os.path.join(REPO, "chipmunk2d_gb300", "_build")
ORACLE_DIR = os.path.join(REPO, "oracle", "_build")
REF_DIR = os.path.join(REPO, "oracle", "_ref")


def reference_headers():
    root = os.environ.get("CHIPMUNK_REF_ROOT") or os.path.join(os.path.dirname(REPO), "reference")
    inc = os.path.join(root, "include")
    return inc if os.path.exists(os.path.join(inc, "chipmunk", "chipmunk.h")) else None


def build(tmp_path, name, libdir, lib, ref_headers=None, program="relink_program.c"):
    gcc = shutil.which("gcc")
    if gcc is None:
        pytest.skip("no C compiler")
    exe = str(tmp_path / name)
    cmd = [gcc, "-std=gnu99", "-O2", "-ffp-contract=off"]
    if ref_headers:
        cmd += ["-DRELINK_REFERENCE_HEADERS", "-I", ref_headers]
    else:
        cmd += ["-I", os.path.join(REPO, "include")]
    cmd += [os.path.join(REPO, "tests", program), "-o", exe, "-L", libdir, "-l" + lib, "-Wl,-rpath," + libdir, "-lm"]
    subprocess.check_call(cmd)
    return exe


def run(exe):
    """(row labels, values) of the program's output: one row per body and
    per query result, the values printed as hexadecimal floats."""
    out = subprocess.run([exe], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300, check=True).stdout
    rows = [ln.split() for ln in out.strip().splitlines()]
    # the shape iteration order must agree exactly: it goes into the labels
    rows = [[" ".join(r)] if r[0] in ("order", "poststep") else r for r in rows]
    ids = [r[0] for r in rows]
    width = max(len(r) for r in rows)
    vals = np.array([[float.fromhex(x) if x.startswith(("0x", "-0x")) else float(x) for x in r[1:]] + [0.0] * (width - len(r))
                     for r in rows])
    return ids, vals


@pytest.mark.parametrize("program", PROGRAMS)
def test_builds_against_the_reference_headers_and_links_the_gpu_library(tmp_path, program):
    """Source and link compatibility: the program compiled with the
    reference's own headers links against libchipmunk_gb300.so."""
    inc = reference_headers()
    if inc is None:
        pytest.skip("reference headers not present on this machine")
    if not os.path.exists(os.path.join(GPU_DIR, "libchipmunk_gb300.so")):
        pytest.skip("libchipmunk_gb300.so not built")
    build(tmp_path, "relink_ref_headers", GPU_DIR, "chipmunk_gb300", ref_headers=inc, program=program)


@pytest.mark.parametrize("program", PROGRAMS)
def test_oracle_matches_the_reference_on_the_program(tmp_path, oracle_lib, program):
    """The same program on the reference library and on the oracle: bit for
    bit, through removals and additions mid-run, caller-placed objects,
    every joint kind, the queries and sleeping."""
    if not os.path.exists(os.path.join(REF_DIR, "libcpref.so")):
        pytest.skip("reference library not built on this machine")
    ids_r, ref = run(build(tmp_path, "relink_ref", REF_DIR, "cpref", program=program))
    ids_o, orc = run(build(tmp_path, "relink_oracle", ORACLE_DIR, "oracle", program=program))
    assert ids_r == ids_o and len(ids_r) > 20
    np.testing.assert_array_equal(orc, ref)


@pytest.mark.gpu
@pytest.mark.parametrize("program", PROGRAMS)
def test_gpu_library_runs_the_program_like_the_oracle(tmp_path, oracle_lib, program):
    """The program linked against libchipmunk_gb300.so runs on the GPU and
    ends where the oracle does.  Two free runs (no state copied between
    them): the last-bit differences of sin/cos compound over the 180 steps,
    so positions and velocities are held to 1e-9 of their magnitude, as in
    the free-run pyramid test."""
    ids_o, orc = run(build(tmp_path, "relink_oracle", ORACLE_DIR, "oracle", program=program))
    ids_g, gpu = run(build(tmp_path, "relink_gpu", GPU_DIR, "chipmunk_gb300", program=program))
    assert ids_g == ids_o
    scale = np.maximum(np.abs(orc).max(axis=0), 1.0)
    err = float((np.abs(gpu - orc) / scale).max())
    print("relinked program: GPU against oracle, worst rel err %.3g" % err)
    assert err <= 1e-9, err


LOCKED_MODES = ["none", "add", "remove", "type", "sleep"]


def run_locked(exe, mode):
    """(exit status, stdout, the first line of stderr) of relink_locked.c."""
    p = subprocess.run([exe, mode], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True, timeout=300)
    err = p.stderr.strip().splitlines()
    return p.returncode, p.stdout, err[0] if err else ""


def check_locked(got, want, mode):
    assert got == want
    status, out, err = got
    assert "locked 1" in out and out.strip().endswith(("after locked 0", "locked 1"))
    if mode == "none":
        assert status == 0 and "after locked 0" in out
    else:
        assert status != 0 and err.startswith("Aborting due to Chipmunk error: "), got


@pytest.mark.parametrize("mode", LOCKED_MODES)
def test_oracle_refuses_edits_while_locked_like_the_reference(tmp_path, oracle_lib, mode):
    """Queries and iterations lock the space (cpSpaceIsLocked reads true in
    their callbacks); an add, a removal, a type change or a sleep made
    there aborts with the reference's message."""
    if not os.path.exists(os.path.join(REF_DIR, "libcpref.so")):
        pytest.skip("reference library not built on this machine")
    ref = run_locked(build(tmp_path, "locked_ref", REF_DIR, "cpref", program="relink_locked.c"), mode)
    orc = run_locked(build(tmp_path, "locked_oracle", ORACLE_DIR, "oracle", program="relink_locked.c"), mode)
    check_locked(orc, ref, mode)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", LOCKED_MODES)
def test_gpu_library_refuses_edits_while_locked(tmp_path, oracle_lib, mode):
    orc = run_locked(build(tmp_path, "locked_oracle", ORACLE_DIR, "oracle", program="relink_locked.c"), mode)
    gpu = run_locked(build(tmp_path, "locked_gpu", GPU_DIR, "chipmunk_gb300", program="relink_locked.c"), mode)
    check_locked(gpu, orc, mode)

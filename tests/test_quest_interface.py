"""CPU: the quest signed-distance C interface (include/gsq_quest.h) keeps the
reference's entry points and error behaviour: the serial build's
QUEST_signed_distance_* symbols of quest/interface/c_fortran/wrapQUEST.h:84-129,
init failing with -1 on a missing or empty file name, and the process aborting
on misuse, as the reference's death tests expect
(quest/tests/quest_signed_distance_interface.cpp:245-335).  Each check runs in
a child process: the interface keeps global state, and misuse ends the process.
No GPU is used (nothing here reaches a query)."""
from __future__ import annotations

import os
import signal
import subprocess
import sys
import textwrap

import pytest

from conftest import ROOT

# the serial-build entry points of wrapQUEST.h:92-129
REFERENCE_ENTRY_POINTS = [
    "QUEST_signed_distance_init_serial", "QUEST_signed_distance_init_serial_bufferify",
    "QUEST_signed_distance_initialized", "QUEST_signed_distance_get_mesh_bounds",
    "QUEST_signed_distance_set_dimension", "QUEST_signed_distance_set_closed_surface",
    "QUEST_signed_distance_set_compute_signs", "QUEST_signed_distance_set_allocator",
    "QUEST_signed_distance_set_verbose", "QUEST_signed_distance_use_shared_memory",
    "QUEST_signed_distance_set_execution_space", "QUEST_signed_distance_evaluate_0",
    "QUEST_signed_distance_evaluate_1", "QUEST_signed_distance_finalize",
]

PRELUDE = """
import ctypes as C
from axom_gb300 import build
build.build()
import axom_gb300
lib = axom_gb300.load()
"""


def run_child(body: str):
    code = PRELUDE + textwrap.dedent(body)
    return subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)


def test_exports_the_reference_entry_points():
    from axom_gb300 import build
    build.build()
    import axom_gb300
    lib = axom_gb300.load()
    header = (ROOT / "include/gsq_quest.h").read_text()
    for name in REFERENCE_ENTRY_POINTS:
        assert name in header and hasattr(lib, name), name


def test_init_failures_and_options_before_init():
    """signed_distance_init("") and ("badfile.stl") return nonzero and leave
    the query uninitialized (quest_signed_distance_interface.cpp:337-349);
    every option can be set before init; a Fortran blank-padded name is
    trimmed."""
    p = run_child("""
        assert not lib.QUEST_signed_distance_initialized()
        assert lib.QUEST_signed_distance_init_serial(b"") != 0
        assert not lib.QUEST_signed_distance_initialized()
        assert lib.QUEST_signed_distance_init_serial(b"badfile.stl") != 0
        assert b"badfile.stl" in lib.gsq_last_error()
        assert not lib.QUEST_signed_distance_initialized()
        name = b"badfile.stl" + b" " * 13
        assert lib.QUEST_signed_distance_init_serial_bufferify(name, len(name)) != 0
        assert b"badfile.stl " not in lib.gsq_last_error()
        lib.QUEST_signed_distance_set_dimension(3)
        lib.QUEST_signed_distance_set_closed_surface(False)
        lib.QUEST_signed_distance_set_compute_signs(True)
        lib.QUEST_signed_distance_set_allocator(-1)
        lib.QUEST_signed_distance_set_verbose(True)
        lib.QUEST_signed_distance_use_shared_memory(True)
        for s in (0, 1, 2):
            lib.QUEST_signed_distance_set_execution_space(s)
        assert lib.gsq_quest_set_precision(7) != 0
        assert lib.gsq_quest_set_precision(0) == 0 and lib.gsq_quest_set_precision(1) == 0
        h = C.c_void_p(1)
        assert lib.gsq_quest_handle(C.byref(h)) == 0 and not h.value
        lib.QUEST_signed_distance_finalize()  # a no-op before init
        assert not lib.QUEST_signed_distance_initialized()
        print("OK")
    """)
    assert p.returncode == 0 and "OK" in p.stdout, p.stdout + p.stderr
    assert "Option is ignored" in p.stderr  # shared memory needs MPI-3


@pytest.mark.parametrize("call,message", [
    ("lib.QUEST_signed_distance_evaluate_0(0.0, 0.0, 0.0)", "must be initialized"),
    ("lib.QUEST_signed_distance_evaluate_1(0.0, 0.0, 0.0, *[C.pointer(C.c_double()) for _ in range(6)])",
     "must be initialized"),
    ("lib.gsq_quest_evaluate_points(None, None, None, 2, None)", "must be initialized"),
    ("lo = (C.c_double * 3)(); lib.QUEST_signed_distance_get_mesh_bounds(lo, lo)", "must be initialized"),
    ("lib.QUEST_signed_distance_set_dimension(2)", "only support 3D"),
    ("lib.QUEST_signed_distance_set_execution_space(5)", "Unsupported execution space"),
])
def test_misuse_aborts_like_the_reference(call, message):
    """evaluate and get_mesh_bounds before init, a dimension other than 3 and
    an unknown execution space end the process (SLIC_ERROR)."""
    p = run_child(f"print('before', flush=True)\n{call}\nprint('after')")
    assert "before" in p.stdout and "after" not in p.stdout, p.stdout + p.stderr
    assert p.returncode == -signal.SIGABRT, (p.returncode, p.stderr)
    assert message in p.stderr, p.stderr


@pytest.fixture(scope="module")
def mocked_c_caller(tmp_path_factory):
    """tests/cpp/quest_check.c linked with libgsq.so and tests/cpp/oracle_double.cpp,
    whose oracle-backed gsq_sdf_* functions take the place of the GPU query."""
    from axom_gb300 import build
    build.build()
    d = tmp_path_factory.mktemp("quest_mock")
    inc, lib_dir = ROOT / "include", ROOT / "axom_gb300"
    subprocess.run(["gcc", "-std=c99", "-O1", f"-I{inc}", "-c", str(ROOT / "tests/cpp/quest_check.c"), "-o",
                    str(d / "qc.o")], check=True)
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fopenmp", f"-I{inc}", "-c",
                    str(ROOT / "tests/cpp/oracle_double.cpp"), "-o", str(d / "qm.o")], check=True)
    exe = d / "quest_mocked"
    subprocess.run(["g++", "-rdynamic", "-fopenmp", str(d / "qc.o"), str(d / "qm.o"), f"-L{lib_dir}", "-lgsq", "-lm",
                    f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    return exe


def test_c_caller_known_answers_on_the_oracle(mocked_c_caller, tmp_path):
    """The interface's logic as built into libgsq.so, over the oracle: the
    reference's plane known answers to 4 ulp, closest points and normals, the
    nodes' bounds, a refused second init, finalize, a blank-padded Fortran name
    and an unsigned re-init."""
    p = subprocess.run([str(mocked_c_caller), str(tmp_path / "plane.stl")], capture_output=True, text=True,
                       timeout=300)
    assert p.returncode == 0 and "OK" in p.stdout, p.stdout + p.stderr


@pytest.mark.parametrize("case,message", [("0", "already initialized"), ("1", "already initialized"),
                                          ("2", "already initialized"), ("3", "already initialized"),
                                          ("4", "buffer is null"), ("5", "already initialized"),
                                          ("6", "already initialized"), ("7", "already initialized")])
def test_misuse_after_init_aborts_on_the_oracle(mocked_c_caller, tmp_path, case, message):
    p = subprocess.run([str(mocked_c_caller), str(tmp_path / "plane.stl"), case], capture_output=True, text=True,
                       timeout=300)
    assert "before" in p.stdout and "after" not in p.stdout, p.stdout + p.stderr
    assert p.returncode == -signal.SIGABRT, (p.returncode, p.stderr)
    assert message in p.stderr, p.stderr

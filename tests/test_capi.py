"""CPU: libgsq.so builds, loads, and exports every symbol include/gsq.h declares.

No compute call needs a GPU here; only argument validation and the host
helpers run.
"""
from __future__ import annotations

import ctypes as C
import re

import numpy as np
import pytest

from conftest import ROOT, assert_bits_equal, golden


@pytest.fixture(scope="module")
def lib():
    from axom_gb300 import build
    build.build()
    import axom_gb300
    return axom_gb300.load()


def declared_functions() -> list[str]:
    names = []
    for h in (ROOT / "include").glob("*.h"):
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**((?:gsq|QUEST)_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("gsq_bvh_build", "gsq_bvh_find_boxes", "gsq_bvh_find_points", "gsq_bvh_find_rays",
                 "gsq_sdf_create", "gsq_sdf_eval"):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"symbols declared but not exported: {missing}"


def test_python_signatures_cover_header():
    import axom_gb300
    bound = {n for n, _, _ in axom_gb300.SIGNATURES}
    missing = [n for n in declared_functions() if n not in bound]
    assert not missing, f"entry points without a Python binding: {missing}"


def test_argument_validation_without_gpu(lib):
    assert lib.gsq_bvh_create(None) == -1
    assert b"null" in lib.gsq_last_error()
    assert lib.gsq_bvh_set_scale_factor(None, 1.0) == -1
    assert lib.gsq_sdf_create(None, None, None, None, 0, None, 0, 3, 1, 1, None, None) == -1
    assert lib.gsq_sdf_eval(None, None, None, None, 1, 1, None, None, None, None) == -1
    assert lib.gsq_free(None) == 0
    assert lib.gsq_version().startswith(b"gsq")


def test_ray_normalize_matches_reference(lib):
    import axom_gb300
    g = golden("bvh_boxes2000")
    assert_bits_equal(axom_gb300.normalize_rays(g["ray_dirs_raw"]), g["ray_dirs"], "ray directions")
    z = axom_gb300.normalize_rays(np.zeros((1, 3)))
    assert np.array_equal(z, [[1.0, 0.0, 0.0]])


def test_opts_defaults(lib):
    import axom_gb300
    o = axom_gb300.SdfOpts()
    assert lib.gsq_sdf_opts_init(C.byref(o)) == 0
    assert o.precision == 0 and o.sort_queries == 1


def test_batch_argument_validation_without_gpu(lib):
    import axom_gb300
    o = axom_gb300.BatchOpts()
    assert lib.gsq_batch_opts_init(C.byref(o)) == 0
    h = C.c_void_p()
    vp = lambda a: C.c_void_p(a.ctypes.data)  # noqa: E731
    voff = np.array([0, 4, 8], np.int64)
    coff = np.array([0, 2, 4], np.int64)
    qoff = np.array([0, 10, 10], np.int64)
    cells = np.zeros(12, np.int32)
    bad_cells = np.array([0, 1, 4], np.int64)
    assert lib.gsq_batch_create(C.byref(h), 2, vp(voff), vp(bad_cells), vp(cells), 3, vp(qoff), 1, 1, None,
                                None) == -1
    assert b"at least 2 cells" in lib.gsq_last_error()
    assert lib.gsq_batch_create(C.byref(h), 0, vp(voff), vp(coff), vp(cells), 3, vp(qoff), 1, 1, None, None) == -1
    assert lib.gsq_batch_create(C.byref(h), 2, vp(voff), vp(coff), vp(cells), 5, vp(qoff), 1, 1, None, None) == -1
    shrinking = np.array([0, 10, 5], np.int64)
    assert lib.gsq_batch_create(C.byref(h), 2, vp(voff), vp(coff), vp(cells), 3, vp(shrinking), 1, 1, None,
                                None) == -1
    o.leaf_size = 2
    assert lib.gsq_batch_create(C.byref(h), 2, vp(voff), vp(coff), vp(cells), 3, vp(qoff), 1, 1, C.byref(o),
                                None) == -1
    assert b"leaf_size" in lib.gsq_last_error()
    o.leaf_size, o.queue_depth = 1, 3
    assert lib.gsq_batch_create(C.byref(h), 2, vp(voff), vp(coff), vp(cells), 3, vp(qoff), 1, 1, C.byref(o),
                                None) == -1
    assert lib.gsq_batch_run(None, None, None, None) == -1
    assert lib.gsq_batch_destroy(None) == 0


def test_callers_compile_and_link(lib, tmp_path):
    """The C++ shim caller and the C99 caller of the quest entry points compile
    against include/ and link libgsq.so (they run in the GPU suite)."""
    import subprocess
    lib_dir = ROOT / "axom_gb300"
    for src, cc in (("shim_check.cpp", ["g++", "-std=c++17"]), ("quest_check.c", ["gcc", "-std=c99"])):
        exe = tmp_path / src.split(".")[0]
        p = subprocess.run(cc + ["-O1", "-Wall", "-Werror", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp" / src),
                                 f"-L{lib_dir}", "-lgsq", "-lm", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)],
                           capture_output=True, text=True)
        assert p.returncode == 0, p.stderr


def test_cpp_shim_known_answers_on_the_oracle(lib, tmp_path):
    """tests/cpp/shim_check.cpp (the reference's BVH, plane, STL, quest
    interface and closest-point known answers through include/gsq.hpp) with
    the GPU entry points taken over by the oracle-backed double
    (tests/cpp/oracle_double.cpp): the shim's host logic on a machine without
    a GPU.  The GPU suite runs the same program on the GPU entry points."""
    import subprocess
    inc, lib_dir = ROOT / "include", ROOT / "axom_gb300"
    objs = []
    for src, flags in (("shim_check.cpp", []), ("oracle_double.cpp", ["-ffp-contract=off", "-fopenmp"])):
        obj = tmp_path / (src.split(".")[0] + ".o")
        subprocess.run(["g++", "-std=c++17", "-O1", *flags, f"-I{inc}", "-c", str(ROOT / "tests/cpp" / src), "-o",
                        str(obj)], check=True)
        objs.append(str(obj))
    exe = tmp_path / "shim_on_oracle"
    subprocess.run(["g++", "-rdynamic", "-fopenmp", *objs, f"-L{lib_dir}", "-lgsq", f"-Wl,-rpath,{lib_dir}", "-o",
                    str(exe)], check=True)
    p = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300, cwd=tmp_path)
    assert p.returncode == 0 and "OK" in p.stdout, p.stdout + p.stderr

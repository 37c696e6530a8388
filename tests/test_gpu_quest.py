"""GPU: the quest signed-distance C interface (include/gsq_quest.h).

* a C99 program written against the reference's shroud entry points
  (tests/cpp/quest_check.c) passes the reference's interface known answers
  (quest/tests/quest_signed_distance_interface.cpp: failing inits, the analytic
  plane to 4 ulp, mesh bounds, finalize, an unsigned re-init);
* the global query over an STL file equals the oracle on the same nodes and
  triangles bit for bit (distances and closest points; unit normals within
  1e-12), through evaluate(x, y, z), evaluate(x, y, z, cp, n) and the array
  form, in both precision forms and every closed / sign combination;
* options set after init, a null bounds buffer and a second mesh init abort
  the process, as the reference's death tests expect (:245-335); these run in
  child processes, which abort on the host only (no kernel is in flight)."""
from __future__ import annotations

import ctypes as C
import signal
import subprocess
import sys
import textwrap

import numpy as np
import pytest

from axom_gb300 import workloads as W
from conftest import ROOT, assert_bits_equal

pytestmark = pytest.mark.gpu


def write_stl(path, v, f):
    """ASCII STL with every coordinate written to round-trip exactly."""
    with open(path, "w") as out:
        out.write("solid quest\n")
        for t in f:
            out.write(" facet normal 0 0 0\n  outer loop\n")
            for i in t:
                out.write("   vertex " + " ".join(repr(float(c)) for c in v[i]) + "\n")
            out.write("  endloop\n endfacet\n")
        out.write("endsolid quest\n")


def test_c_caller_known_answers(gsq, tmp_path):
    exe = tmp_path / "quest_check"
    lib_dir = ROOT / "axom_gb300"
    subprocess.run(["gcc", "-std=c99", "-O2", f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/quest_check.c"),
                    f"-L{lib_dir}", "-lgsq", "-lm", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], check=True)
    p = subprocess.run([str(exe), str(tmp_path / "plane.stl")], capture_output=True, text=True, timeout=300,
                       cwd=tmp_path)
    assert p.returncode == 0, p.stdout + p.stderr
    assert "OK" in p.stdout


def test_global_query_matches_oracle(gsq, port, tmp_path):
    lib = gsq.load()
    v, f = W.displaced_icosphere(3, 5)
    path = tmp_path / "ico3.stl"
    write_stl(path, v, f)
    nodes, cells = gsq.read_stl(path)
    q = np.concatenate([W.uniform_queries(v, 200, 1), W.near_surface_queries(v, f, 200, 2), v[:40],
                        W.uniform_queries(v, 20, 3, factor=6.0)])
    qx, qy, qz = (np.ascontiguousarray(q[:, k]) for k in range(3))
    outs = [C.c_double() for _ in range(6)]
    try:
        for precision in (0, 1):
            for closed, sign in ((True, True), (False, True), (True, False)):
                what = f"precision {precision}, closed {closed}, sign {sign}"
                assert lib.gsq_quest_set_precision(precision) == 0
                lib.QUEST_signed_distance_set_closed_surface(closed)
                lib.QUEST_signed_distance_set_compute_signs(sign)
                assert lib.QUEST_signed_distance_init_serial(str(path).encode()) == 0, lib.gsq_last_error()
                assert lib.QUEST_signed_distance_initialized()
                h = port.sdf(nodes[:, 0], nodes[:, 1], nodes[:, 2], cells, closed, sign)
                d_ref, cp_ref, n_ref = port.sdf_eval(h, q, True, True)
                d0 = np.array([lib.QUEST_signed_distance_evaluate_0(float(a), float(b), float(c)) for a, b, c in q])
                assert_bits_equal(d0, d_ref, f"evaluate(x, y, z), {what}")
                d1, cp, nr = np.empty(len(q)), np.empty((len(q), 3)), np.empty((len(q), 3))
                for i, (a, b, c) in enumerate(q):
                    d1[i] = lib.QUEST_signed_distance_evaluate_1(float(a), float(b), float(c),
                                                                 *[C.byref(o) for o in outs])
                    cp[i] = [o.value for o in outs[:3]]
                    nr[i] = [o.value for o in outs[3:]]
                assert_bits_equal(d1, d_ref, f"evaluate(x, y, z, cp, n), {what}")
                assert_bits_equal(cp, cp_ref, f"closest points, {what}")
                np.testing.assert_allclose(nr, n_ref, rtol=0, atol=1e-12)
                phi = np.full(len(q), np.nan)
                lib.gsq_quest_evaluate_points(qx.ctypes.data, qy.ctypes.data, qz.ctypes.data, len(q),
                                              phi.ctypes.data)
                assert_bits_equal(phi, d_ref, f"evaluate(x, y, z, n, phi), {what}")
                lo, hi = (C.c_double * 3)(), (C.c_double * 3)()
                lib.QUEST_signed_distance_get_mesh_bounds(lo, hi)
                assert_bits_equal(np.array(lo[:]), nodes.min(0), "mesh bounds lo")
                assert_bits_equal(np.array(hi[:]), nodes.max(0), "mesh bounds hi")
                handle = C.c_void_p()
                assert lib.gsq_quest_handle(C.byref(handle)) == 0 and handle.value
                assert lib.QUEST_signed_distance_init_serial(str(path).encode()) != 0  # already initialized
                lib.QUEST_signed_distance_finalize()
                assert not lib.QUEST_signed_distance_initialized()
    finally:
        lib.QUEST_signed_distance_finalize()
        lib.QUEST_signed_distance_set_closed_surface(True)
        lib.QUEST_signed_distance_set_compute_signs(True)
        lib.gsq_quest_set_precision(1)


@pytest.mark.parametrize("call,message", [
    ("lib.QUEST_signed_distance_set_closed_surface(True)", "already initialized"),
    ("lib.QUEST_signed_distance_set_dimension(3)", "already initialized"),
    ("lib.QUEST_signed_distance_set_verbose(True)", "already initialized"),
    ("lib.QUEST_signed_distance_set_execution_space(0)", "already initialized"),
    ("hi = (C.c_double * 3)(); lib.QUEST_signed_distance_get_mesh_bounds(None, hi)", "buffer is null"),
    ("lib.gsq_quest_init_mesh(None, None, None, 0, None, 0)", "already been initialized"),
])
def test_misuse_after_init_aborts(gsq, tmp_path, call, message):
    path = tmp_path / "ico2.stl"
    write_stl(path, *W.displaced_icosphere(2, 5))
    code = textwrap.dedent(f"""
        import ctypes as C
        import axom_gb300
        lib = axom_gb300.load()
        assert lib.QUEST_signed_distance_init_serial({str(path)!r}.encode()) == 0, lib.gsq_last_error()
        assert lib.QUEST_signed_distance_evaluate_0(0.0, 0.0, 0.0) < 0  # inside the closed surface
        print("before", flush=True)
        {call}
        print("after")
    """)
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=300, cwd=ROOT)
    assert "before" in p.stdout and "after" not in p.stdout, p.stdout + p.stderr
    assert p.returncode == -signal.SIGABRT, (p.returncode, p.stderr)
    assert message in p.stderr, p.stderr

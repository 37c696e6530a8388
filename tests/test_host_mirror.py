"""CPU: the Python mirror's host plumbing (axom_gb300.BVH, SignedDistance,
ClosestPoint: argument staging, AoS and SoA strides, output shapes, the
candidate CSR copies) over libgsq.so with the GPU entry points taken over by
the oracle-backed double (tests/cpp/oracle_double.cpp, put in front of the
library's entry points in a child process), checked bit for bit against the
golden fixtures the reference made.  The GPU suite runs the same classes on the
GPU entry points."""
from __future__ import annotations

import subprocess
import sys
import textwrap

from conftest import ROOT

CHECKS = """
import ctypes as C
import numpy as np
import axom_gb300 as gsq

G = {root!r} + "/tests/golden/"

# The mirror calls libgsq.so through its own handle, so the double's entry
# points are put in front of the library's here, with the same signatures.
real, double = gsq.load(), C.CDLL({double!r})


class Merged:
    def __getattr__(self, name):
        try:
            f = getattr(double, name)
        except AttributeError:
            return getattr(real, name)
        g = getattr(real, name)
        f.restype, f.argtypes = g.restype, g.argtypes
        return f


gsq._lib = Merged()


def same(a, b, what):
    a, b = np.asarray(a), np.asarray(b)
    assert a.shape == b.shape and a.dtype == b.dtype, (what, a.shape, b.shape, a.dtype, b.dtype)
    assert np.array_equal(a.view(np.uint8), b.view(np.uint8)), what


g = np.load(G + "bvh_boxes2000.npz")
for scale, tag in ((1.000123, "s"), (1.0, "u")):
    b = gsq.BVH(g["boxes"], scale_factor=scale)
    assert b.get_scale_factor() == scale and b.num_leaves() == len(g["boxes"])
    lo, hi = b.get_bounds()
    same(np.concatenate([lo, hi]), g[tag + "_bvh_bounds"], "bounds")
    for key, res in (("fb", b.find_bounding_boxes(g["query_boxes"])), ("fp", b.find_points(g["points"])),
                     ("fr", b.find_rays(g["ray_origins"], g["ray_dirs"]))):
        for name, arr in zip(("offsets", "counts", "candidates"), res):
            same(arr, g[tag + "_" + key + "_" + name], key + " " + name)
same(gsq.normalize_rays(g["ray_dirs_raw"]), g["ray_dirs"], "ray normalisation")

for name in ("sdf_uvsphere", "sdf_ico3", "sdf_ico3_open", "sdf_ico3_unsigned", "sdf_quad12"):
    f = np.load(G + name + ".npz")
    sd = gsq.SignedDistance(f["vertices"], f["cells"], bool(f["watertight"]), bool(f["sign"]))
    d, cp, nr = sd.compute_distances(f["queries"], closest=True, normals=True)
    same(d, f["dist"], name + " distance")
    same(cp, f["closest"], name + " closest")
    np.testing.assert_allclose(nr, f["normals"], rtol=0, atol=1e-12)
    same(sd.compute_distances(f["queries"]), f["dist"], name + " distance only")
    q = np.ascontiguousarray(f["queries"])
    out = np.empty(len(q))
    sd.compute_distances_soa(q[:, 0].copy(), q[:, 1].copy(), q[:, 2].copy(), out)
    same(out, f["dist"], name + " SoA")
    lo, hi = sd.get_mesh_bounds()
    same(np.concatenate([lo, hi]), f["mesh_bounds"], name + " bounds")
    assert sd.compute_distances(q[:0]).shape == (0,)

c = np.load(G + "cp_points3000.npz")
cpq = gsq.ClosestPoint(c["points"], c["domains"])
for tag, thr in (("all", None), ("thr", 0.05)):
    if thr is not None:
        cpq.set_distance_threshold(thr)
    for got, key in zip(cpq.compute_closest_points(c["queries"]), ("idx", "dom", "pos", "dist")):
        same(got, c[tag + "_" + key], "closest object point " + tag + " " + key)
print("OK")
"""


def test_python_mirror_on_the_oracle(tmp_path):
    from axom_gb300 import build
    build.build()
    double = tmp_path / "liboracle_double.so"
    subprocess.run(["g++", "-std=c++17", "-O1", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared",
                    f"-I{ROOT / 'include'}", str(ROOT / "tests/cpp/oracle_double.cpp"), "-o", str(double)], check=True)
    code = textwrap.dedent(CHECKS.format(root=str(ROOT), double=str(double)))
    p = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert p.returncode == 0 and "OK" in p.stdout, p.stdout + p.stderr

"""Generates the golden fixtures in tests/golden/ by running the reference.

The reference is axom's own SEQ path compiled from its sources by
oracle/build_ref.py (oracle/_ref/libaxom_ref.so); it exists only where the
reference tree is mounted, so the fixtures are committed and the GPU tests
compare against them without it.  Inputs come from axom_gb300.workloads with
fixed seeds.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import oracle  # noqa: E402
from axom_gb300 import workloads as W  # noqa: E402

OUT = Path(__file__).resolve().parent


def csr(off, cnt, cand):
    return dict(offsets=off.astype(np.int32), counts=cnt.astype(np.int32), candidates=cand.astype(np.int32))


def bvh_fixture(R):
    boxes = W.random_boxes(2000, 1)
    qboxes = W.random_boxes(2000, 2)
    pts = W.rng(5).uniform(0.0, 1.0, size=(2000, 3))
    ro = W.rng(6).uniform(-0.2, 1.2, size=(500, 3))
    rd = W.rng(7).normal(size=(500, 3))
    rd[::9, 0] = 0.0  # axis-parallel rays exercise the near-zero direction branch
    out = {"boxes": boxes, "query_boxes": qboxes, "points": pts, "ray_origins": ro, "ray_dirs_raw": rd}
    for scale, tag in ((1.000123, "s"), (1.0, "u")):
        it = R.internals(boxes, scale)
        for k in ("codes", "perm", "lchild", "rchild", "parents", "inner", "bounds"):
            out[f"{tag}_{k}"] = it[k]
        h = R.bvh(boxes, scale)
        out[f"{tag}_bvh_bounds"] = R.bounds(h)
        for k, v in csr(*R.find_boxes(h, qboxes)).items():
            out[f"{tag}_fb_{k}"] = v
        for k, v in csr(*R.find_points(h, pts)).items():
            out[f"{tag}_fp_{k}"] = v
        off, cnt, cand, dirs = R.find_rays(h, ro, rd)
        for k, v in csr(off, cnt, cand).items():
            out[f"{tag}_fr_{k}"] = v
        out["ray_dirs"] = dirs
    np.savez_compressed(OUT / "bvh_boxes2000.npz", **out)


def bvh_dense_fixture(R):
    """Queries that hit: over the same 2,000 boxes as bvh_boxes2000, 1,000
    query boxes 5-400x larger than the inserted ones (sides uniform in
    [0.05, 0.4]), points inside or on the corners of inserted boxes, and rays
    aimed at inserted boxes' centres (some along the axes), so the reference's
    candidate lists, and their order, are dense."""
    boxes = W.random_boxes(2000, 1)
    g = W.rng(40)
    c = g.uniform(0.0, 1.0, size=(1000, 3))
    side = g.uniform(0.05, 0.4, size=(1000, 3))
    qboxes = np.concatenate([c - 0.5 * side, c + 0.5 * side], axis=1)
    pick = g.integers(0, 2000, size=1500)
    lo, hi = boxes[pick, :3], boxes[pick, 3:]
    pts = lo + g.uniform(0.0, 1.0, size=(1500, 3)) * (hi - lo)
    pts[:300] = lo[:300]          # exactly on a corner (inclusive containment)
    pts[300:500] = hi[300:500]
    pick = g.integers(0, 2000, size=800)
    ro = g.uniform(-0.2, 1.2, size=(800, 3))
    target = 0.5 * (boxes[pick, :3] + boxes[pick, 3:])
    rd = target - ro
    ro[:150] = target[:150]       # axis-parallel rays from a box centre
    rd[:150] = 0.0
    rd[np.arange(150), np.arange(150) % 3] = np.where(np.arange(150) % 2 == 0, 1.0, -1.0)
    out = {"boxes": boxes, "query_boxes": qboxes, "points": pts, "ray_origins": ro, "ray_dirs_raw": rd}
    for scale, tag in ((1.000123, "s"), (1.0, "u")):
        h = R.bvh(boxes, scale)
        for k, v in csr(*R.find_boxes(h, qboxes)).items():
            out[f"{tag}_fb_{k}"] = v
        for k, v in csr(*R.find_points(h, pts)).items():
            out[f"{tag}_fp_{k}"] = v
        off, cnt, cand, dirs = R.find_rays(h, ro, rd)
        for k, v in csr(off, cnt, cand).items():
            out[f"{tag}_fr_{k}"] = v
        out["ray_dirs"] = dirs
    np.savez_compressed(OUT / "bvh_dense.npz", **out)


def sdf_fixture(R, name, v, f, q, watertight=True, sign=True):
    h = R.sdf(v[:, 0], v[:, 1], v[:, 2], f, watertight, sign)
    d, cp, nr = R.sdf_eval(h, q, True, True)
    nb, nl = R.sdf_counts(h, q)
    np.savez_compressed(OUT / f"{name}.npz", vertices=v, cells=f, queries=q, dist=d, closest=cp, normals=nr,
                        box_tests=nb, leaf_tests=nl, mesh_bounds=R.mesh_bounds(h), watertight=watertight, sign=sign)


def cp_fixture(R):
    """The local closest-point query of DistributedClosestPoint: object points
    (a sixth of them exact duplicates, so ties occur) with domain ids; query
    points uniform in the 1.2x box plus some exactly on object points; results
    without a threshold and with threshold 0.05 (squared 0.0025)."""
    r = W.rng(21)
    pts = r.uniform(0.0, 1.0, size=(3000, 3))
    pts[2500:] = pts[:500]
    dom = r.integers(0, 5, size=3000).astype(np.int32)
    q = r.uniform(-0.1, 1.1, size=(3000, 3))
    q[:300] = pts[1000:1300]
    h = R.cp(pts, dom)
    out = {"points": pts, "domains": dom, "queries": q}
    for tag, thr in (("all", float(np.finfo(np.float64).max)), ("thr", 0.05 * 0.05)):
        idx, d, pos, dist = R.cp_query(h, q, thr)
        out.update({f"{tag}_idx": idx, f"{tag}_dom": d, f"{tag}_pos": pos, f"{tag}_dist": dist})
    np.savez_compressed(OUT / "cp_points3000.npz", **out)


def main():
    if oracle.build_reference() is None:
        raise SystemExit("reference sources not found; fixtures can only be made where they are mounted")
    R = oracle.Ref()
    if sys.argv[1:] == ["cp"]:  # only the closest-point fixture
        cp_fixture(R)
        return
    if sys.argv[1:] == ["bvh_dense"]:  # only the dense candidate fixture
        bvh_dense_fixture(R)
        return
    cp_fixture(R)
    bvh_fixture(R)
    bvh_dense_fixture(R)
    # UV sphere of quest_signed_distance.cpp:86-169 on its 16^3 grid over the
    # sphere box expanded by 2.0
    v, f = W.uv_sphere()
    lo, hi = v.min(0) - 2.0, v.max(0) + 2.0
    sdf_fixture(R, "sdf_uvsphere", v, f, W.uniform_grid(lo, hi, 16))
    # displaced level-3 icosphere, uniform + near-surface queries
    v, f = W.displaced_icosphere(3, 1234)
    sdf_fixture(R, "sdf_ico3", v, f, W.mixed_queries(v, f, 4000, 11))
    # open surface (not watertight), and unsigned
    keep = f[:, 0] % 7 != 0
    sdf_fixture(R, "sdf_ico3_open", v, f[keep], W.uniform_queries(v, 1500, 12), watertight=False)
    sdf_fixture(R, "sdf_ico3_unsigned", v, f, W.uniform_queries(v, 1500, 13), sign=False)
    # quad surface (cells split into two triangles, SD:651-658)
    vq, fq = W.quad_sphere(12)
    vq = W.displace(vq, 5)
    hq = R.sdf(vq[:, 0], vq[:, 1], vq[:, 2], fq)
    qq = W.mixed_queries(vq, fq[:, :3], 2000, 14)
    d, cp, nr = R.sdf_eval(hq, qq, True, True)
    np.savez_compressed(OUT / "sdf_quad12.npz", vertices=vq, cells=fq, queries=qq, dist=d, closest=cp, normals=nr,
                        mesh_bounds=R.mesh_bounds(hq), watertight=True, sign=True)
    print("fixtures written to", OUT)


if __name__ == "__main__":
    main()

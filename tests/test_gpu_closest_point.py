"""GPU: the local closest-point query of quest::DistributedClosestPoint.

Both forms (FP64 and FP32-certified nodes) must equal the reference's outputs
(golden fixture) and the oracle (live, larger clouds) bit for bit: index,
domain, position and distance, NaN patterns included.  Tolerance: bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

import axom_gb300
from conftest import assert_bits_equal, golden

pytestmark = pytest.mark.gpu

PRECISIONS = [axom_gb300.PRECISION_FP64, axom_gb300.PRECISION_MIXED]


def check(got, want):
    for x, y, what in zip(got, want, ("index", "domain", "position", "distance")):
        assert_bits_equal(np.asarray(x), np.asarray(y), what)


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("tag", ["all", "thr"])
def test_closest_point_matches_golden(gsq, precision, tag):
    g = golden("cp_points3000")
    cp = gsq.ClosestPoint(g["points"], g["domains"])
    if tag == "thr":
        cp.set_distance_threshold(0.05)
    got = cp.compute_closest_points(g["queries"], precision=precision)
    check(got, tuple(g[f"{tag}_{k}"] for k in ("idx", "dom", "pos", "dist")))


@pytest.mark.parametrize("precision", PRECISIONS)
@pytest.mark.parametrize("n", [0, 1, 2, 200_000])
def test_closest_point_matches_oracle(gsq, port, precision, n):
    r = np.random.default_rng(50 + n)
    pts = r.uniform(-5, 5, (n, 3))
    if n > 2:
        pts[n // 3:n // 3 + 1000] = pts[:1000]  # duplicates: ties
    dom = r.integers(0, 17, n).astype(np.int32)
    q = r.uniform(-6, 6, (100_000, 3))
    if n:
        q[:500] = pts[:min(n, 500)].repeat(500 // min(n, 500) + 1, 0)[:500]
    cp = gsq.ClosestPoint(pts, dom)
    h = port.cp(pts, dom)
    for t in (None, 0.2):
        thr = float(np.finfo(np.float64).max) if t is None else t * t
        if t is not None:
            cp.set_distance_threshold(t)
        check(cp.compute_closest_points(q, precision=precision), port.cp_query(h, q, thr, threads=8))


def test_closest_point_device_arrays(gsq, port):
    import torch
    r = np.random.default_rng(7)
    pts = r.normal(size=(50_000, 3))
    q = r.normal(size=(20_000, 3)) * 1.5
    cp = gsq.ClosestPoint(torch.from_numpy(pts).cuda())
    idx, dom, pos, dist = cp.compute_closest_points(torch.from_numpy(q).cuda())
    want = port.cp_query(port.cp(pts), q, threads=8)
    check((idx.cpu().numpy(), dom.cpu().numpy(), pos.cpu().numpy(), dist.cpu().numpy()), want)


def test_closest_point_ties_at_scale(gsq, port):
    """The 655,362 vertices of the level-8 mesh as object points; 2M queries:
    uniform in the 1.2x box, and at midpoints of mesh edges (two object points
    at equal distance up to rounding, so the strict "closer" test and the
    first-found rule decide).  Mixed against FP64 over every output, and a
    sample against the oracle, bit for bit."""
    import torch
    from axom_gb300 import workloads as W
    v, f = W.displaced_icosphere(8, 1234)
    r = np.random.default_rng(12)
    e = f[r.integers(0, f.shape[0], 1 << 20), :2]
    q = np.concatenate([W.uniform_queries(v, 1 << 20, 13), 0.5 * (v[e[:, 0]] + v[e[:, 1]])])
    qd = torch.from_numpy(q).cuda()
    cp = gsq.ClosestPoint(v)
    mixed = cp.compute_closest_points(qd, precision=axom_gb300.PRECISION_MIXED)
    fp64 = cp.compute_closest_points(qd, precision=axom_gb300.PRECISION_FP64)
    for x, y, what in zip(mixed, fp64, ("index", "domain", "position", "distance")):
        assert_bits_equal(x.cpu().numpy(), y.cpu().numpy(), what)
    idx = np.concatenate([np.arange(0, 1 << 20, 97), (1 << 20) + np.arange(0, 1 << 20, 97)])
    want = port.cp_query(port.cp(v), q[idx], threads=16)
    check(tuple(x.cpu().numpy()[idx] for x in mixed), want)
